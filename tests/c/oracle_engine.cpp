// The device-resident ABI calls the CLI makes, restated on the CPU oracle.
//
// TEST INFRASTRUCTURE ONLY.  tests/test_cli_host_cpu.py links the CLI front
// end (ddevol_gb300/cli/tpgp_gb_cli.c) against this file, the library's
// host-only record code (ddevol_gb300/csrc/checkpoint.cu) and the oracle, so
// that the CLI's own logic -- options, CSV rows, checkpoint cadence, restarts,
// walltime pauses, cap stops -- runs on a machine without a GPU.  The
// product library never contains it; the oracle's Strang step is bitwise the
// device engine's (the GPU suite checks that), so the CLI's outputs here are
// the outputs it gives on the device.
#include <cmath>
#include <cstring>
#include <new>

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

}  // extern "C"
