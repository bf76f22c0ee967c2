// The device-resident ABI calls that the CLI and the serving loop make,
// restated on the CPU oracle.
//
// TEST INFRASTRUCTURE ONLY.  tests/test_cli_host_cpu.py links the CLI front
// end (ddevol_gb300/cli/tpgp_gb_cli.c) against this file, the library's
// host-only record code (ddevol_gb300/csrc/checkpoint.cu) and the oracle, so
// that the CLI's own logic -- options, CSV rows, checkpoint cadence, restarts,
// walltime pauses, cap stops -- runs on a machine without a GPU;
// tests/test_serve_host_cpu.py does the same for the continuous-batching
// loop (ddevol_gb300/csrc/serve.cu) over the batch calls below.  The
// product library never contains it; the oracle's Strang step is bitwise the
// device engine's (the GPU suite checks that), so the outputs here are the
// outputs the same host code gives on the device.
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <new>
#include <vector>

#include "../../include/tpgp_gb300.h"
#include "../../oracle/tpgp_oracle.h"

extern "C" double orc_strang_bound(const orc_term* terms, size_t count, double dt);

struct tpgp_gb_context {
    int device;
};
struct tpgp_gb_map {
    orc_map m;
};

static_assert(sizeof(tpgp_gb_term) == sizeof(orc_term), "term layouts differ");
static_assert(sizeof(tpgp_gb_ledger) == sizeof(orc_ledger), "ledger layouts differ");

extern "C" {

tpgp_gb_context* tpgp_gb_create(int device, char* error, size_t cap) {
    if (error && cap) error[0] = '\0';
    return new (std::nothrow) tpgp_gb_context{device};
}

void tpgp_gb_destroy(tpgp_gb_context* ctx) { delete ctx; }

tpgp_gb_options tpgp_gb_default_options(void) {
    tpgp_gb_options o;
    std::memset(&o, 0, sizeof(o));
    o.exact_ledger = 1;  // the library's default: the reference's sequential ledger
    o.use_graphs = 1;
    return o;
}

tpgp_gb_status tpgp_gb_map_create(tpgp_gb_context*, size_t n_spins, tpgp_gb_map** out, char*,
                                  size_t) {
    auto* m = new (std::nothrow) tpgp_gb_map();
    if (!m || orc_map_from_arrays(&m->m, n_spins, nullptr, nullptr, 0) != ORC_OK) {
        delete m;
        return TPGP_GB_ENOMEM;
    }
    *out = m;
    return TPGP_GB_OK;
}

void tpgp_gb_map_destroy(tpgp_gb_map* m) {
    if (!m) return;
    orc_map_free(&m->m);
    delete m;
}

size_t tpgp_gb_map_len(const tpgp_gb_map* m) { return m ? m->m.len : 0; }
size_t tpgp_gb_map_spins(const tpgp_gb_map* m) { return m ? m->m.n_spins : 0; }

tpgp_gb_status tpgp_gb_map_upload(tpgp_gb_map* m, const uint64_t* keys, const double* values,
                                  size_t len, char*, size_t) {
    const size_t n = m->m.n_spins;
    orc_map_free(&m->m);
    return (tpgp_gb_status)orc_map_from_arrays(&m->m, n, keys, values, len);
}

tpgp_gb_status tpgp_gb_map_download(const tpgp_gb_map* m, uint64_t* keys, double* values,
                                    size_t capacity, size_t* len, char*, size_t) {
    if (capacity < m->m.len) return TPGP_GB_EINVAL;
    std::memcpy(keys, m->m.keys, m->m.len * m->m.n_words * sizeof(uint64_t));
    std::memcpy(values, m->m.values, m->m.len * sizeof(double));
    *len = m->m.len;
    return TPGP_GB_OK;
}

tpgp_gb_status tpgp_gb_strang_step(tpgp_gb_map* m, const tpgp_gb_term* terms, size_t count,
                                   double dt, const tpgp_gb_options* o, tpgp_gb_ledger* ledger,
                                   char* error, size_t cap) {
    const int st = orc_strang_step(&m->m, reinterpret_cast<const orc_term*>(terms), count, dt,
                                   o->threshold, o->max_terms, o->max_drop_l2, 1,
                                   reinterpret_cast<orc_ledger*>(ledger));
    if (error && cap) error[0] = '\0';
    return (tpgp_gb_status)st;
}

double tpgp_gb_strang_bound(const tpgp_gb_term* terms, size_t count, double dt) {
    return orc_strang_bound(reinterpret_cast<const orc_term*>(terms), count, dt);
}

tpgp_gb_status tpgp_gb_single_sum(const tpgp_gb_map* m, unsigned pauli, double* sum) {
    *sum = orc_single_sum(&m->m, pauli);
    return TPGP_GB_OK;
}

// tpgp_map_l2 (engine/src/tpgp_rev.c:266-271): a long-double sum of squares
tpgp_gb_status tpgp_gb_map_l2(const tpgp_gb_map* m, double* l2) {
    long double s = 0;
    for (size_t k = 0; k < m->m.len; ++k) s += (long double)m->m.values[k] * m->m.values[k];
    *l2 = (double)std::sqrt(s);
    return TPGP_GB_OK;
}

// ---- batches: independent maps stepped together (tpgp_gb_batch_*)

struct tpgp_gb_batch {
    std::vector<orc_map> maps;
    std::vector<std::vector<tpgp_gb_term>> terms;
    std::vector<double> dt;
    std::vector<tpgp_gb_options> opts;
    std::vector<tpgp_gb_ledger> ledgers;
    std::vector<int> failed;
    double last_ms = 0;
    size_t last_terms = 0;
};

tpgp_gb_status tpgp_gb_batch_create(tpgp_gb_context*, size_t n, const size_t* n_spins,
                                    tpgp_gb_batch** out, char*, size_t) {
    if (!n || !n_spins || !out) return TPGP_GB_EINVAL;
    auto* bt = new (std::nothrow) tpgp_gb_batch();
    if (!bt) return TPGP_GB_ENOMEM;
    bt->maps.resize(n);
    for (size_t i = 0; i < n; ++i) orc_map_from_arrays(&bt->maps[i], n_spins[i], nullptr, nullptr, 0);
    bt->terms.resize(n);
    bt->dt.assign(n, 0.0);
    bt->opts.assign(n, tpgp_gb_default_options());
    bt->ledgers.assign(n, tpgp_gb_ledger{});
    bt->failed.assign(n, 0);
    *out = bt;
    return TPGP_GB_OK;
}

void tpgp_gb_batch_destroy(tpgp_gb_batch* bt) {
    if (!bt) return;
    for (auto& m : bt->maps) orc_map_free(&m);
    delete bt;
}

// a new operator starts a new solve: fresh ledger, no failure
tpgp_gb_status tpgp_gb_batch_upload(tpgp_gb_batch* bt, size_t item, const uint64_t* keys,
                                    const double* values, size_t len, char*, size_t) {
    if (!bt || item >= bt->maps.size()) return TPGP_GB_EINVAL;
    const size_t n = bt->maps[item].n_spins;
    orc_map_free(&bt->maps[item]);
    const int st = orc_map_from_arrays(&bt->maps[item], n, keys, values, len);
    bt->failed[item] = 0;
    bt->ledgers[item] = tpgp_gb_ledger{};
    return (tpgp_gb_status)st;
}

tpgp_gb_status tpgp_gb_batch_set_terms(tpgp_gb_batch* bt, size_t item, const tpgp_gb_term* terms,
                                       size_t count, double dt, const tpgp_gb_options* o, char*,
                                       size_t) {
    if (!bt || item >= bt->maps.size() || (!terms && count) || !o || !std::isfinite(dt))
        return TPGP_GB_EINVAL;
    if (dt * 0.5 * 2 != dt) return TPGP_GB_ENUMERIC;
    bt->terms[item].assign(terms, terms + count);
    bt->dt[item] = dt;
    bt->opts[item] = *o;
    return TPGP_GB_OK;
}

// `steps` Strang steps of every healthy item with terms and a non-empty map;
// fid_sums[k * n + i] the item's single sum of X after step k (NaN when
// failed or idle)
tpgp_gb_status tpgp_gb_batch_step(tpgp_gb_batch* bt, size_t steps, double* fid_sums, char*, size_t) {
    if (!bt) return TPGP_GB_EINVAL;
    const auto t0 = std::chrono::steady_clock::now();
    const size_t n = bt->maps.size();
    bt->last_terms = 0;
    for (size_t k = 0; k < steps; ++k)
        for (size_t i = 0; i < n; ++i) {
            orc_map& m = bt->maps[i];
            double fid = std::numeric_limits<double>::quiet_NaN();
            if (!bt->failed[i] && !bt->terms[i].empty() && m.len) {
                bt->last_terms += m.len * 2 * bt->terms[i].size();
                const tpgp_gb_options& o = bt->opts[i];
                const int st = orc_strang_step(
                    &m, reinterpret_cast<const orc_term*>(bt->terms[i].data()), bt->terms[i].size(),
                    bt->dt[i], o.threshold, o.max_terms, o.max_drop_l2, 1,
                    reinterpret_cast<orc_ledger*>(&bt->ledgers[i]));
                if (st) bt->failed[i] = st;
                else fid = orc_single_sum(&m, 1);
            }
            if (fid_sums) fid_sums[k * n + i] = fid;
        }
    bt->last_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return TPGP_GB_OK;
}

int tpgp_gb_batch_item_status(const tpgp_gb_batch* bt, size_t item) {
    return bt && item < bt->failed.size() ? bt->failed[item] : (int)TPGP_GB_EINVAL;
}

tpgp_gb_status tpgp_gb_batch_ledger(const tpgp_gb_batch* bt, size_t item, tpgp_gb_ledger* out) {
    if (!bt || item >= bt->ledgers.size() || !out) return TPGP_GB_EINVAL;
    *out = bt->ledgers[item];
    return TPGP_GB_OK;
}

double tpgp_gb_batch_last_elapsed_ms(const tpgp_gb_batch* bt) { return bt ? bt->last_ms : 0.0; }
size_t tpgp_gb_batch_last_terms(const tpgp_gb_batch* bt) { return bt ? bt->last_terms : 0; }
size_t tpgp_gb_batch_last_launches(const tpgp_gb_batch*) { return 0; }

}  // extern "C"
