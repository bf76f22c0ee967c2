/*
 * The reference-facing branch backend (include/tpgp_cuda_rev.h) driven from
 * C, the way the reference engine drives its CUDA backend.
 *
 * Links libtpgp_gb300.so through include/tpgp_cuda_rev.h only, and the CPU
 * oracle (oracle/tpgp_oracle.h, test infrastructure) as the engine around
 * it: with the oracle's branch hook pointed at tpgp_cuda_branches, every
 * rotation of a Strang step takes its raw children from the GPU and sorts,
 * merges, thresholds and books them on the host -- the flow of DDevol's
 * rotate_product with backend TPGP_CUDA (engine/src/tpgp_rev.c:622-640,
 * statuses mapped as at :635-638).  Checked here:
 *
 *   1. the argument and status contract of tpgp_cuda_branches (engine/
 *      include/tpgp_cuda_rev.h:25-48; engine/src/cuda_rev.cu:180-203) and of
 *      tpgp_cuda_create for invalid devices;
 *   2. raw children bitwise equal to the oracle's branch (keys, values,
 *      radii with and without enclosure) for key widths of 1, 2, 3 and 32
 *      words, every generator pair, random sites;
 *   3. Strang trajectories of J1-J2 rings (6, 40 and 70 spins, from the sum
 *      of X over all sites, thresholds 0 and 1e-5) with the GPU as the
 *      branch backend, map and ledger bitwise equal to the oracle's own;
 *   4. the same trajectories through tpgp_cuda_branches_static;
 *   5. two threads sharing one context.
 *
 * Exit status: 0 when every check passed, 1 when one failed, 77 when no
 * device is visible (the library then refuses to create a context and has
 * no CPU substitute); with --require-device a missing device is 1.
 */
#include <float.h>
#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "tpgp_cuda_rev.h"
#include "tpgp_oracle.h"

static unsigned g_checks, g_failures;

#define EXPECT(cond, ...)                                                   \
    do {                                                                    \
        ++g_checks;                                                         \
        if (!(cond)) {                                                      \
            ++g_failures;                                                   \
            fprintf(stderr, "check failed (line %d): ", __LINE__);          \
            fprintf(stderr, __VA_ARGS__);                                   \
            fputc('\n', stderr);                                            \
        }                                                                   \
    } while (0)

/* splitmix64: seeded inputs that do not depend on the C library's rand() */
static uint64_t next_random(uint64_t *state) {
    uint64_t z = (*state += UINT64_C(0x9E3779B97F4A7C15));
    z = (z ^ (z >> 30)) * UINT64_C(0xBF58476D1CE4E5B9);
    z = (z ^ (z >> 27)) * UINT64_C(0x94D049BB133111EB);
    return z ^ (z >> 31);
}

static double uniform(uint64_t *state) { return (double)(next_random(state) >> 11) * 0x1p-53; }

static int same_bits(const void *a, const void *b, size_t bytes) { return !memcmp(a, b, bytes); }

/* ------------------------------------------------------------ 1. contract */

typedef struct {
    const char *what;
    tpgp_cuda_status want;
    int null_context, null_keys, words, spins, i, j, qi, qj, enclose, out_keys_alias;
    size_t count;
    double c, rc;
    uint64_t key;
    double value;
} contract_case;

static void check_contract(tpgp_cuda_context *ctx) {
    const double nan = NAN, inf = INFINITY;
    /* one valid call: 2 spins, 1 word, ZZ on sites 0 and 1, c = 0.6, s = 0.8 */
    const contract_case base = {"valid", TPGP_CUDA_OK, 0, 0, 1, 2, 0, 1, 3, 3, 1, 0,
                                1, 0.6, 0.0, 1, 1.0};
    contract_case cases[20];
    size_t n = 0;
#define CASE(label, status, field, value_)          \
    do {                                            \
        cases[n] = base;                            \
        cases[n].what = label;                      \
        cases[n].want = status;                     \
        cases[n].field = value_;                    \
        ++n;                                        \
    } while (0)
    CASE("NULL context", TPGP_CUDA_EINVAL, null_context, 1);
    CASE("NULL input keys", TPGP_CUDA_EINVAL, null_keys, 1);
    CASE("byte count overflow", TPGP_CUDA_EINVAL, count, SIZE_MAX);
    CASE("word count not ceil(spins/32)", TPGP_CUDA_EINVAL, words, 2);
    CASE("one spin", TPGP_CUDA_EINVAL, spins, 1);
    CASE("equal sites", TPGP_CUDA_EINVAL, j, 0);
    CASE("site beyond the spins", TPGP_CUDA_EINVAL, j, 2);
    CASE("Pauli label 4", TPGP_CUDA_EINVAL, qi, 4);
    CASE("NaN cosine", TPGP_CUDA_EINVAL, c, nan);
    CASE("infinite radius", TPGP_CUDA_EINVAL, rc, inf);
    CASE("negative radius", TPGP_CUDA_EINVAL, rc, -1.0);
    CASE("enclose flag 2", TPGP_CUDA_EINVAL, enclose, 2);
    CASE("output keys alias the input keys", TPGP_CUDA_EINVAL, out_keys_alias, 1);
    CASE("bits above the last site", TPGP_CUDA_EINVAL, key, 16);
    CASE("NaN coefficient", TPGP_CUDA_ENUMERIC, value, nan);
    CASE("infinite coefficient", TPGP_CUDA_ENUMERIC, value, inf);
    CASE("a commuting (identity) key with an infinite coefficient", TPGP_CUDA_ENUMERIC, key, 0);
    cases[n - 1].value = inf;
    CASE("child overflow (DBL_MAX * 2)", TPGP_CUDA_ENUMERIC, value, DBL_MAX);
    cases[n - 1].c = 2.0;
    CASE("valid call after the failures", TPGP_CUDA_OK, enclose, 1);
#undef CASE
    for (size_t k = 0; k < n; ++k) {
        const contract_case *t = cases + k;
        uint64_t key = t->key, out_keys[2] = {0, 0};
        double value = t->value, out_values[2] = {0, 0}, out_radii[2] = {0, 0};
        char error[256] = "untouched";
        tpgp_cuda_status st = tpgp_cuda_branches(
            t->null_context ? NULL : ctx, t->null_keys ? NULL : &key, &value, t->count,
            (size_t)t->words, (size_t)t->spins, (size_t)t->i, (size_t)t->j, (unsigned)t->qi,
            (unsigned)t->qj, t->c, 0.8, t->rc, 0.0, t->enclose, t->out_keys_alias ? &key : out_keys,
            out_values, out_radii, error, sizeof(error));
        EXPECT(st == t->want, "%s: status %d, expected %d (%s)", t->what, (int)st, (int)t->want,
               error);
        if (t->want != TPGP_CUDA_OK)
            EXPECT(error[0] != '\0' && strcmp(error, "untouched") != 0,
                   "%s: no message for a failure", t->what);
        else
            EXPECT(error[0] == '\0', "%s: message on success: %s", t->what, error);
    }
    /* the valid ZZ call on X_0: anticommuting, children (X_0, 0.6) and
     * (Y_0 Z_1, +-0.8) */
    {
        uint64_t key = 1, out_keys[2];
        double value = 1.0, out_values[2], out_radii[2];
        char error[128];
        tpgp_cuda_status st = tpgp_cuda_branches(ctx, &key, &value, 1, 1, 2, 0, 1, 3, 3, 0.6, 0.8,
                                                 0.0, 0.0, 0, out_keys, out_values, out_radii,
                                                 error, sizeof(error));
        EXPECT(st == TPGP_CUDA_OK && out_keys[0] == 1 && out_keys[1] == (1 ^ 3 ^ (3u << 2)) &&
                   out_values[0] == 0.6 && fabs(out_values[1]) == 0.8,
               "ZZ on X_0: status %d keys %llx %llx values %g %g", (int)st,
               (unsigned long long)out_keys[0], (unsigned long long)out_keys[1], out_values[0],
               out_values[1]);
    }
    /* empty batch: NULL arrays accepted */
    {
        char error[64];
        EXPECT(tpgp_cuda_branches(ctx, NULL, NULL, 0, 1, 2, 0, 1, 3, 3, 0.6, 0.8, 0, 0, 0, NULL,
                                  NULL, NULL, error, sizeof(error)) == TPGP_CUDA_OK,
               "empty batch with NULL arrays");
    }
    {
        char error[128];
        EXPECT(tpgp_cuda_create(-1, error, sizeof(error)) == NULL && error[0],
               "create(-1) must fail with a message");
        EXPECT(tpgp_cuda_create(INT_MAX, error, sizeof(error)) == NULL && error[0],
               "create(INT_MAX) must fail with a message");
        EXPECT(!strcmp(tpgp_cuda_device_name(NULL), "unavailable"), "device name of NULL");
    }
}

/* --------------------------------------------------- 2. raw branch parity */

/* A random valid key of `spins` sites: 2 bits per site, padding bits zero. */
static void random_key(uint64_t *state, size_t spins, size_t words, uint64_t *key) {
    for (size_t w = 0; w < words; ++w) key[w] = next_random(state);
    const size_t rem = spins % 32;
    if (rem) key[words - 1] &= (UINT64_C(1) << (2 * rem)) - 1;
}

static int compare_batch(tpgp_cuda_context *ctx, uint64_t *state, size_t spins, size_t count,
                         unsigned qi, unsigned qj, int enclose, int use_static) {
    const size_t words = (spins + 31) / 32;
    uint64_t *keys = malloc(count * words * sizeof(uint64_t));
    double *values = malloc(count * sizeof(double));
    uint64_t *gk = malloc(2 * count * words * sizeof(uint64_t));
    uint64_t *ok = malloc(2 * count * words * sizeof(uint64_t));
    double *gv = malloc(2 * count * sizeof(double)), *ov = malloc(2 * count * sizeof(double));
    double *gr = malloc(2 * count * sizeof(double)), *orad = malloc(2 * count * sizeof(double));
    int good = keys && values && gk && ok && gv && ov && gr && orad;
    if (good) {
        for (size_t k = 0; k < count; ++k) {
            random_key(state, spins, words, keys + k * words);
            /* magnitudes over many binades, both signs, a few exact zeros */
            double m = ldexp(uniform(state) + 0.5, (int)(next_random(state) % 80) - 40);
            values[k] = (next_random(state) % 64 == 0) ? 0.0 : (next_random(state) & 1 ? m : -m);
        }
        const size_t i = next_random(state) % spins;
        size_t j = next_random(state) % (spins - 1);
        if (j >= i) ++j;
        const double angle = 6.283185307179586 * uniform(state);  /* [0, 2 pi) */
        const double c = cos(angle), s = sin(angle);
        const double rc = enclose ? 0x1p-53 : 0.0, rs = enclose ? 0x1p-52 : 0.0;
        char error[256];
        tpgp_cuda_status st =
            use_static ? tpgp_cuda_branches_static(0, keys, values, count, words, spins, i, j, qi,
                                                   qj, c, s, rc, rs, enclose, gk, gv, gr, error,
                                                   sizeof(error))
                       : tpgp_cuda_branches(ctx, keys, values, count, words, spins, i, j, qi, qj,
                                            c, s, rc, rs, enclose, gk, gv, gr, error,
                                            sizeof(error));
        int ost = orc_branches(keys, values, count, words, spins, i, j, qi, qj, c, s, rc, rs,
                               enclose, ok, ov, orad);
        good = st == TPGP_CUDA_OK && ost == 0 &&
               same_bits(gk, ok, 2 * count * words * sizeof(uint64_t)) &&
               same_bits(gv, ov, 2 * count * sizeof(double)) &&
               same_bits(gr, orad, 2 * count * sizeof(double));
        if (!good)
            fprintf(stderr, "branch mismatch: spins %zu sites %zu/%zu labels %u/%u enclose %d "
                    "static %d status %d/%d %s\n", spins, i, j, qi, qj, enclose, use_static,
                    (int)st, ost, error);
    }
    free(keys), free(values), free(gk), free(ok), free(gv), free(ov), free(gr), free(orad);
    return good;
}

static void check_branch_parity(tpgp_cuda_context *ctx) {
    const size_t spin_counts[] = {2, 31, 32, 33, 64, 70, 96, 1000};
    uint64_t state = UINT64_C(0x5eed0001);
    unsigned batches = 0, good = 0;
    for (size_t a = 0; a < sizeof(spin_counts) / sizeof(spin_counts[0]); ++a)
        for (unsigned q = 0; q < 16; ++q) {
            const size_t count = spin_counts[a] == 1000 ? 257 : 3001;
            good += (unsigned)compare_batch(ctx, &state, spin_counts[a], count, q >> 2, q & 3u,
                                            (int)(q & 1u), 0);
            ++batches;
        }
    /* the allocation-free entry point on a subset */
    for (unsigned q = 0; q < 16; ++q, ++batches)
        good += (unsigned)compare_batch(ctx, &state, 64, 2049, q >> 2, q & 3u, (int)(q & 1u), 1);
    EXPECT(good == batches, "%u of %u random branch batches bitwise equal", good, batches);
}

/* ------------------------------------- 3-4. engine flow on the GPU backend */

typedef struct {
    tpgp_cuda_context *ctx;  /* NULL: the allocation-free entry point on device 0 */
    double *radii;
    size_t radii_cap;
    unsigned calls;
} gpu_backend;

static int gpu_branch(void *user, const uint64_t *keys, const double *values, size_t count,
                      size_t words, size_t spins, size_t i, size_t j, unsigned qi, unsigned qj,
                      double c, double s, uint64_t *out_keys, double *out_values) {
    gpu_backend *b = user;
    if (2 * count > b->radii_cap) {
        free(b->radii);
        b->radii_cap = 4 * count;
        b->radii = malloc(b->radii_cap * sizeof(double));
        if (!b->radii) {
            b->radii_cap = 0;
            return ORC_ENOMEM;
        }
    }
    char error[256];
    tpgp_cuda_status st =
        b->ctx ? tpgp_cuda_branches(b->ctx, keys, values, count, words, spins, i, j, qi, qj, c, s,
                                    0.0, 0.0, 0, out_keys, out_values, b->radii, error,
                                    sizeof(error))
               : tpgp_cuda_branches_static(0, keys, values, count, words, spins, i, j, qi, qj, c,
                                           s, 0.0, 0.0, 0, out_keys, out_values, b->radii, error,
                                           sizeof(error));
    ++b->calls;
    if (st != TPGP_CUDA_OK) fprintf(stderr, "branch backend: %s\n", error);
    /* the engine's status mapping (engine/src/tpgp_rev.c:635-638) */
    return st == TPGP_CUDA_OK         ? ORC_OK
           : st == TPGP_CUDA_ENOMEM   ? ORC_ENOMEM
           : st == TPGP_CUDA_ENUMERIC ? ORC_ENUMERIC
                                      : ORC_EBACKEND;
}

/* Periodic J1-J2 ring, reference edge order: for each site the (s, s+1)
 * then the (s, s+2) edge, each as ZZ d/2, XX -d/4, YY -d/4 with d = 2 J. */
static size_t ring_terms(size_t spins, double j1, double j2, orc_term *out) {
    size_t n = 0;
    for (size_t s = 0; s < spins; ++s)
        for (size_t range = 1; range <= 2; ++range) {
            const double d = 2.0 * (range == 1 ? j1 : j2);
            const unsigned labels[3] = {3, 1, 2};
            const double h[3] = {d / 2, -d / 4, -d / 4};
            for (int g = 0; g < 3; ++g) {
                orc_term t = {s, (s + range) % spins, labels[g], labels[g], h[g], n};
                out[n++] = t;
            }
        }
    return n;
}

/* The sum of X over all sites, keys ascending. */
static int global_x(orc_map *m, size_t spins) {
    const size_t words = (spins + 31) / 32;
    uint64_t *keys = calloc(spins * words, sizeof(uint64_t));
    double *values = malloc(spins * sizeof(double));
    int st = ORC_ENOMEM;
    if (keys && values) {
        for (size_t s = 0; s < spins; ++s) {
            keys[s * words + s / 32] = UINT64_C(1) << (2 * (s % 32));
            values[s] = 1.0;
        }
        st = orc_map_from_arrays(m, spins, keys, values, spins);
    }
    free(keys), free(values);
    return st;
}

static int same_map(const orc_map *a, const orc_map *b) {
    return a->len == b->len && a->n_words == b->n_words &&
           same_bits(a->keys, b->keys, a->len * a->n_words * sizeof(uint64_t)) &&
           same_bits(a->values, b->values, a->len * sizeof(double));
}

static int same_ledger(const orc_ledger *x, const orc_ledger *y) {
    return same_bits(&x->dropped_l1, &y->dropped_l1, sizeof(double)) &&
           same_bits(&x->dropped_l2, &y->dropped_l2, sizeof(double)) &&
           same_bits(&x->dropped_l2_squared, &y->dropped_l2_squared, sizeof(double)) &&
           same_bits(&x->arithmetic_l2, &y->arithmetic_l2, sizeof(double)) &&
           x->rotations == y->rotations && x->removal_events == y->removal_events &&
           x->peak_terms == y->peak_terms;
}

static void check_trajectory(tpgp_cuda_context *ctx, size_t spins, double threshold, int steps) {
    orc_term terms[6 * 128];
    const size_t nt = ring_terms(spins, 1.0, 0.125, terms);
    orc_map cpu, gpu;
    orc_ledger lc, lg;
    memset(&lc, 0, sizeof(lc));
    memset(&lg, 0, sizeof(lg));
    if (global_x(&cpu, spins) || global_x(&gpu, spins)) {
        EXPECT(0, "out of host memory");
        return;
    }
    gpu_backend backend = {ctx, NULL, 0, 0};
    const double dt = 1.0 / 64;
    for (int step = 0; step < steps; ++step) {
        orc_set_branch_backend(NULL, NULL);
        int sc = orc_strang_step(&cpu, terms, nt, dt, threshold, 0, 0.0, 1, &lc);
        orc_set_branch_backend(gpu_branch, &backend);
        int sg = orc_strang_step(&gpu, terms, nt, dt, threshold, 0, 0.0, 1, &lg);
        orc_set_branch_backend(NULL, NULL);
        EXPECT(sc == ORC_OK && sg == ORC_OK, "%zu spins step %d: statuses %d / %d", spins, step,
               sc, sg);
        EXPECT(same_map(&cpu, &gpu) && same_ledger(&lc, &lg),
               "%zu spins, threshold %g, %s, step %d: map (%zu / %zu terms) or ledger differs",
               spins, threshold, ctx ? "context" : "allocation-free", step, cpu.len, gpu.len);
        EXPECT(orc_single_sum(&cpu, 1) == orc_single_sum(&gpu, 1), "FID sums differ");
    }
    EXPECT(backend.calls == lg.rotations, "the backend served %u of %zu rotations",
           backend.calls, lg.rotations);
    printf("%3zu spins, threshold %-6g %-16s %d steps: %zu terms, %zu rotations on the GPU "
           "backend, map and ledger bitwise the oracle's\n",
           spins, threshold, ctx ? "context" : "allocation-free", steps, gpu.len, lg.rotations);
    free(backend.radii);
    orc_map_free(&cpu);
    orc_map_free(&gpu);
}

/* ------------------------------------------------- 5. concurrent callers */

typedef struct {
    tpgp_cuda_context *ctx;
    uint64_t seed;
    int good;
} thread_job;

static void *thread_main(void *arg) {
    thread_job *job = arg;
    job->good = 1;
    for (unsigned q = 0; q < 16; ++q)
        job->good &= compare_batch(job->ctx, &job->seed, 40, 5003, q >> 2, q & 3u, 1, 0);
    return NULL;
}

static void check_concurrent(tpgp_cuda_context *ctx) {
    thread_job jobs[2] = {{ctx, UINT64_C(0xa11ce), 0}, {ctx, UINT64_C(0xb0b), 0}};
    pthread_t threads[2];
    int started = 0;
    for (int t = 0; t < 2; ++t)
        if (!pthread_create(threads + t, NULL, thread_main, jobs + t)) ++started;
    for (int t = 0; t < started; ++t) pthread_join(threads[t], NULL);
    EXPECT(started == 2 && jobs[0].good && jobs[1].good, "two threads on one context");
}

int main(int argc, char **argv) {
    const int require = argc == 2 && !strcmp(argv[1], "--require-device");
    if (argc > 2 || (argc == 2 && !require)) {
        fprintf(stderr, "usage: %s [--require-device]\n", argv[0]);
        return 2;
    }
    EXPECT(tpgp_cuda_compiled() == 1, "tpgp_cuda_compiled() must be 1");
    char error[256];
    tpgp_cuda_context *ctx = tpgp_cuda_create(0, error, sizeof(error));
    if (!ctx) {
        /* no device: the library reports it and offers no CPU path */
        printf("no CUDA device: %s (no CPU substitute)\n", error[0] ? error : "(no message)");
        return g_failures ? 1 : require ? 1 : 77;
    }
    printf("device: %s\n", tpgp_cuda_device_name(ctx));
    check_contract(ctx);
    check_branch_parity(ctx);
    check_trajectory(ctx, 6, 0.0, 3);
    check_trajectory(ctx, 6, 1e-5, 3);
    check_trajectory(ctx, 40, 1e-5, 2);
    check_trajectory(ctx, 70, 1e-5, 1);
    check_trajectory(NULL, 6, 1e-5, 3);
    check_trajectory(NULL, 40, 1e-5, 2);
    check_concurrent(ctx);
    tpgp_cuda_destroy(ctx);
    printf("%u checks, %u failed\n", g_checks, g_failures);
    return g_failures ? 1 : 0;
}
