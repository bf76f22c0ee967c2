// Continuous-batching server for FID solves (include/tpgp_gb300.h,
// tpgp_gb_serve).  Host-only code over the public batch ABI: slots are the
// items of one tpgp_gb_batch; every tick is one batched Strang step of all
// admitted solves.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/tpgp_gb300.h"

namespace {

double seconds_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// device arena bytes per map term for w-word keys: three map buffers, two
// child buffers, removed values, and the doubling slack of the arena
double arena_bytes_per_term(int w) { return 2.0 * (5.0 * (8 * w + 8) + 8.0); }

void widen_keys(const uint64_t* keys, size_t len, size_t from_w, size_t to_w,
                std::vector<uint64_t>* out) {
    out->assign(len * to_w, 0);
    for (size_t k = 0; k < len; ++k)
        for (size_t w = 0; w < from_w; ++w) (*out)[k * to_w + w] = keys[k * from_w + w];
}

}  // namespace

extern "C" tpgp_gb_status tpgp_gb_serve(tpgp_gb_context* ctx, const tpgp_gb_request* req,
                                        size_t n, const size_t slots[3], size_t memory_budget,
                                        double* fids, tpgp_gb_response* resp,
                                        tpgp_gb_serve_stats* stats, char* error, size_t cap) {
    if (error && cap) error[0] = 0;
    if (!ctx || (!req && n) || !slots || !resp) return TPGP_GB_EINVAL;
    // slot layout: slots[0] of 32 spins, slots[1] of 64, slots[2] of 96
    std::vector<size_t> slot_spins;
    for (int w = 0; w < 3; ++w)
        for (size_t k = 0; k < slots[w]; ++k) slot_spins.push_back(32 * (size_t)(w + 1));
    const size_t n_slots = slot_spins.size();
    if (!n_slots) return TPGP_GB_EINVAL;
    for (size_t r = 0; r < n; ++r) {
        if (!req[r].n_spins || req[r].n_spins > 96 || (req[r].len && (!req[r].keys || !req[r].values)) ||
            (req[r].count && !req[r].terms))
            return TPGP_GB_EINVAL;
        if (req[r].n_spins > 32 * (slots[0] ? 1 : 0) && req[r].n_spins > 64 * (slots[1] ? 1 : 0) &&
            req[r].n_spins > 96 * (slots[2] ? 1 : 0)) {
            if (error && cap) std::snprintf(error, cap, "No slot is wide enough for request %zu.", r);
            return TPGP_GB_EINVAL;
        }
    }
    tpgp_gb_batch* bt = nullptr;
    tpgp_gb_status st = tpgp_gb_batch_create(ctx, n_slots, slot_spins.data(), &bt, error, cap);
    if (st) return st;
    std::vector<size_t> fid_off(n + 1, 0);
    for (size_t r = 0; r < n; ++r) fid_off[r + 1] = fid_off[r] + req[r].steps;
    std::vector<long> slot_req(n_slots, -1);     // request in the slot, -1 if free
    std::vector<size_t> done_steps(n, 0);
    std::vector<double> projected(n, 0.0);
    double peak_sum[3] = {0, 0, 0};
    size_t peak_cnt[3] = {0, 0, 0};
    double mem_in_use = 0.0;
    tpgp_gb_serve_stats acc;
    std::memset(&acc, 0, sizeof(acc));
    size_t next = 0, finished = 0;
    std::vector<double> tick_fids(n_slots, 0.0);
    std::vector<uint64_t> wide;
    for (size_t r = 0; r < n; ++r) {
        std::memset(&resp[r], 0, sizeof(resp[r]));
        resp[r].admitted = resp[r].finished = std::nan("");
    }
    const auto t0 = std::chrono::steady_clock::now();
    while (finished < n) {
        const double now = seconds_since(t0);
        // admission: in arrival order; a request that cannot be placed waits
        // (later requests of other widths may still go ahead of it)
        size_t active = 0;
        for (size_t k = 0; k < n_slots; ++k) active += slot_req[k] >= 0;
        for (size_t r = next; r < n && req[r].arrival <= now; ++r) {
            if (!std::isnan(resp[r].admitted)) continue;
            size_t w_need = (req[r].n_spins + 31) / 32;
            long slot = -1;
            for (size_t w = w_need; w <= 3 && slot < 0; ++w)
                for (size_t k = 0; k < n_slots; ++k)
                    if (slot_req[k] < 0 && slot_spins[k] == 32 * w) {
                        slot = (long)k;
                        break;
                    }
            if (slot < 0) continue;
            const int wi = (int)(slot_spins[slot] / 32) - 1;
            const double proj_terms = peak_cnt[wi] ? peak_sum[wi] / peak_cnt[wi] : 1e4;
            const double bytes = proj_terms * arena_bytes_per_term(wi + 1);
            if (active > 0 && mem_in_use + bytes > (double)memory_budget) continue;
            widen_keys(req[r].keys, req[r].len, (req[r].n_spins + 31) / 32, slot_spins[slot] / 32,
                       &wide);
            st = tpgp_gb_batch_upload(bt, (size_t)slot, wide.data(), req[r].values, req[r].len,
                                      error, cap);
            if (st == TPGP_GB_OK)
                st = tpgp_gb_batch_set_terms(bt, (size_t)slot, req[r].terms, req[r].count, req[r].dt,
                                             &req[r].options, error, cap);
            resp[r].admitted = seconds_since(t0);
            resp[r].slot = (size_t)slot;
            resp[r].slot_spins = slot_spins[slot];
            if (st || req[r].steps == 0) {
                // rejected at admission (invalid request) or nothing to do
                resp[r].status = (int)st;
                resp[r].finished = resp[r].admitted;
                ++finished;
                tpgp_gb_batch_set_terms(bt, (size_t)slot, nullptr, 0, 0.5, &req[r].options, nullptr, 0);
                continue;
            }
            slot_req[slot] = (long)r;
            projected[r] = bytes;
            mem_in_use += bytes;
            ++active;
        }
        while (next < n && !std::isnan(resp[next].admitted)) ++next;
        if (active == 0) {
            // idle: wait for the next arrival
            double wait = 1e-3;
            for (size_t r = next; r < n; ++r)
                if (std::isnan(resp[r].admitted)) {
                    wait = std::max(0.0, req[r].arrival - seconds_since(t0));
                    break;
                }
            std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.05)));
            continue;
        }
        // one tick: a Strang step of every admitted solve
        st = tpgp_gb_batch_step(bt, 1, tick_fids.data(), error, cap);
        if (st) {
            tpgp_gb_batch_destroy(bt);
            return st;
        }
        acc.busy_seconds += tpgp_gb_batch_last_elapsed_ms(bt) / 1e3;
        acc.ticks += 1;
        acc.terms += tpgp_gb_batch_last_terms(bt);
        acc.launches += tpgp_gb_batch_last_launches(bt);
        acc.max_active = std::max(acc.max_active, active);
        const double t_tick = seconds_since(t0);
        for (size_t k = 0; k < n_slots; ++k) {
            const long r = slot_req[k];
            if (r < 0) continue;
            const int item_status = tpgp_gb_batch_item_status(bt, k);
            if (item_status == 0) {
                if (fids) fids[fid_off[r] + done_steps[r]] = tick_fids[k];
                resp[r].fid_last = tick_fids[k];
                ++done_steps[r];
            }
            if (item_status != 0 || done_steps[r] == req[r].steps) {
                tpgp_gb_ledger led;
                tpgp_gb_batch_ledger(bt, k, &led);
                resp[r].status = item_status;
                resp[r].finished = t_tick;
                resp[r].peak_terms = led.peak_terms;
                const int wi = (int)(slot_spins[k] / 32) - 1;
                peak_sum[wi] += (double)std::max<size_t>(led.peak_terms, 1);
                peak_cnt[wi] += 1;
                mem_in_use -= projected[r];
                slot_req[k] = -1;
                ++finished;
                // free the slot: no terms, so the next ticks skip it
                tpgp_gb_batch_set_terms(bt, k, nullptr, 0, 0.5, &req[r].options, nullptr, 0);
            }
        }
    }
    acc.wall_seconds = seconds_since(t0);
    if (stats) *stats = acc;
    tpgp_gb_batch_destroy(bt);
    return TPGP_GB_OK;
}
