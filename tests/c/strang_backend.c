/*
 * A device-resident Strang step for DDevol's own tpgp_map, as a maintainer
 * would add it beside tpgp_strang_step (engine/src/tpgp_rev.c:776-809): the
 * map goes up, one step runs on the GB300, the map comes back in the
 * engine's layout, the ledger is the engine's ledger.
 *
 * Built only against the reference checkout (`make -C oracle dropin`): it
 * includes the reference's engine/include/tpgp_rev.h and links its engine,
 * compiled from its own sources, together with libtpgp_gb300.so through
 * include/tpgp_gb300.h.  main() runs the 16-spin J1-J2 ring from X_0 for a
 * few steps with both steps and compares maps and ledgers bit for bit (the
 * reference's own test_cuda_trajectory_rev.c check, for the device-resident
 * engine).  Exit 0: equal; 1: a difference or a failure; 77: no device.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "tpgp_gb300.h"
#include "tpgp_rev.h"

/* One accepted Strang step of `m` on the GPU; the contract of
 * tpgp_strang_step.  `gm` is a device map of m->n_spins spins, created once. */
static tpgp_status gb_strang_step(tpgp_gb_map *gm, tpgp_map *m, const tpgp_term *terms, size_t n,
                                  double dt, const tpgp_options *o, tpgp_ledger *l) {
    char err[256];
    tpgp_gb_options go = tpgp_gb_default_options(); /* exact ledger: the engine's own sums */
    go.threshold = o->threshold;
    go.max_terms = o->max_terms;
    go.max_drop_l2 = o->max_drop_l2;
    /* tpgp_term / tpgp_ledger and tpgp_gb_term / tpgp_gb_ledger share layouts */
    tpgp_gb_status s = tpgp_gb_map_upload(gm, m->keys, m->values, m->len, err, sizeof err);
    if (!s)
        s = tpgp_gb_strang_step(gm, (const tpgp_gb_term *)terms, n, dt, &go, (tpgp_gb_ledger *)l,
                                err, sizeof err);
    if (s) {
        fprintf(stderr, "device step: %s\n", err);
        return (tpgp_status)s; /* same status numbering */
    }
    const size_t len = tpgp_gb_map_len(gm);
    if (len > m->capacity) { /* the engine's storage is malloc'd: grow it in place */
        uint64_t *k = realloc(m->keys, len * m->n_words * sizeof(uint64_t));
        if (k) m->keys = k;
        double *v = realloc(m->values, len * sizeof(double));
        if (v) m->values = v;
        if (!k || !v) return TPGP_ENOMEM;
        m->capacity = len;
    }
    return (tpgp_status)tpgp_gb_map_download(gm, m->keys, m->values, m->capacity, &m->len, err,
                                             sizeof err);
}

static int same_bits(const void *a, const void *b, size_t n) { return !memcmp(a, b, n); }

static int same_ledger(const tpgp_ledger *x, const tpgp_ledger *y) {
    return same_bits(&x->dropped_l1, &y->dropped_l1, sizeof(double)) &&
           same_bits(&x->dropped_l2, &y->dropped_l2, sizeof(double)) &&
           same_bits(&x->dropped_l2_squared, &y->dropped_l2_squared, sizeof(double)) &&
           same_bits(&x->arithmetic_l2, &y->arithmetic_l2, sizeof(double)) &&
           x->rotations == y->rotations && x->removal_events == y->removal_events &&
           x->peak_terms == y->peak_terms && x->arithmetic_enclosed == y->arithmetic_enclosed;
}

int main(void) {
    enum { N = 16 };
    char err[256];
    tpgp_gb_context *ctx = tpgp_gb_create(0, err, sizeof err);
    if (!ctx) {
        printf("no GB300 device: %s (no CPU substitute)\n", err);
        return 77;
    }
    /* the benchmark ring: d(nn) = 1, d(nnn) = 1/8 as ZZ d, XX -d/2, YY -d/2 */
    tpgp_term terms[6 * N];
    size_t count = 0;
    for (size_t i = 0; i < N; i++)
        for (size_t range = 1; range <= 2; range++) {
            const double d = range == 1 ? 1.0 : 0.125;
            const unsigned q[3] = {3, 1, 2};
            const double h[3] = {d, -d / 2, -d / 2};
            for (int g = 0; g < 3; g++) {
                tpgp_term t = {i, (i + range) % N, q[g], q[g], h[g], count};
                terms[count++] = t;
            }
        }
    tpgp_map cpu = {0}, gpu = {0}; /* clone frees its destination's storage first */
    uint64_t x0 = 1; /* X on site 0 */
    if (tpgp_map_init(&cpu, N) || tpgp_map_add(&cpu, &x0, 1.0) || tpgp_map_clone(&gpu, &cpu))
        return 1;
    tpgp_options o = tpgp_default_options();
    o.threshold = 1e-6;
    tpgp_ledger lc, lg;
    tpgp_ledger_init(&lc, 0);
    tpgp_ledger_init(&lg, 0);
    tpgp_gb_map *gm = NULL;
    if (tpgp_gb_map_create(ctx, N, &gm, err, sizeof err))
        return 1;
    int bad = 0;
    for (int step = 0; step < 30 && !bad; step++) {
        const tpgp_status a = tpgp_strang_step(&cpu, terms, count, 0.01, &o, &lc);
        const tpgp_status b = gb_strang_step(gm, &gpu, terms, count, 0.01, &o, &lg);
        bad = a || b || cpu.len != gpu.len ||
              !same_bits(cpu.keys, gpu.keys, cpu.len * cpu.n_words * sizeof(uint64_t)) ||
              !same_bits(cpu.values, gpu.values, cpu.len * sizeof(double)) ||
              !same_ledger(&lc, &lg);
        if (bad)
            fprintf(stderr, "step %d differs (statuses %d/%d, %zu/%zu terms)\n", step + 1, a, b,
                    cpu.len, gpu.len);
    }
    if (!bad)
        printf("30 steps, %zu terms: map and ledger bitwise the engine's\n", gpu.len);
    tpgp_gb_map_destroy(gm);
    tpgp_gb_destroy(ctx);
    tpgp_map_free(&cpu);
    tpgp_map_free(&gpu);
    return bad;
}
