/*
 * CPU oracle for the Pauli-propagation branch step.
 *
 * TEST INFRASTRUCTURE ONLY. This file restates, in plain C, the reference
 * engine's CPU algorithm for one secular two-spin rotation of a sparse Pauli
 * map (DDevol engine/src/tpgp_rev.c).  It is the parity oracle for the CUDA
 * path and the CPU baseline timed by bench.py; no product code path links or
 * calls it.  Only tests/, __graft_entry__.smoke() and bench.py load it.
 *
 * Parity is pinned: tests/golden/make_golden.py runs the reference's own
 * engine (compiled from its sources by oracle/Makefile into oracle/_ref/) on
 * seeded inputs and stores the results under tests/golden/; the CPU test
 * suite checks this oracle against those fixtures bit for bit.
 *
 * Arithmetic is IEEE binary64, round-to-nearest, compiled without fast-math
 * and without FMA contraction (-ffp-contract=off), as the reference requires
 * (engine/CMakeLists.txt:47).
 *
 * Map layout (engine/include/tpgp_rev.h:25-29): keys[k*n_words + w], two
 * bits per site (I=0, X=1, Y=2, Z=3), site s in word s/32 at bit 2*(s%32);
 * keys strictly ascending with the highest word most significant
 * (engine/src/tpgp_rev.c:64-72); no stored zeros.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "tpgp_oracle.h"

/* Directed-rounding helpers: tpgp_rev.c:25-42. */
static double up_add(double a, double b) {
    if (a == 0)
        return b;
    if (b == 0)
        return a;
    return nextafter(a + b, INFINITY);
}
static double up_mul(double a, double b) {
    if (a == 0 || b == 0)
        return 0;
    return nextafter(a * b, INFINITY);
}
static double rounding_radius(double x) {
    if (!isfinite(x))
        return INFINITY;
    double above = fabs(nextafter(x, INFINITY) - x), below = fabs(x - nextafter(x, -INFINITY));
    return above > below ? above : below;
}

/* Multi-word key order, highest word most significant: tpgp_rev.c:64-72. */
static int key_order(const uint64_t *a, const uint64_t *b, size_t words) {
    for (size_t w = words; w-- > 0;) {
        if (a[w] != b[w])
            return a[w] < b[w] ? -1 : 1;
    }
    return 0;
}
static unsigned site_symbol(const uint64_t *key, size_t site) {
    return (unsigned)(key[site / 32] >> (2 * (site % 32))) & 3u;
}
/* Exponent of i in Q*P for single-site Paulis: tpgp_rev.c:414-417. */
static unsigned phase_of(unsigned q, unsigned p) {
    if (!q || !p || q == p)
        return 0;
    /* cyclic X->Y->Z->X gives +i (exponent 1), anticyclic gives -i (3) */
    return ((q % 3) + 1 == p) ? 1u : 3u;
}
static int anticommutes(unsigned q, unsigned p) { return q && p && q != p; }

void orc_trig(double h, double duration, double *c, double *s) {
    /* tpgp_rev.c:528-532: x evaluated as (2*h)*duration, host libm. */
    double x = 2 * h * duration;
    *c = cos(x);
    *s = sin(x);
}

void orc_map_free(orc_map *m) {
    if (!m)
        return;
    free(m->keys);
    free(m->values);
    memset(m, 0, sizeof(*m));
}

/* Builds a map from caller arrays (copied).  No validation beyond sizes:
 * the caller states the invariants it wants checked. */
int orc_map_from_arrays(orc_map *m, size_t n_spins, const uint64_t *keys, const double *values,
                        size_t len) {
    memset(m, 0, sizeof(*m));
    if (!n_spins)
        return ORC_EINVAL;
    m->n_spins = n_spins;
    m->n_words = (n_spins + 31) / 32;
    size_t cap = len ? len : 1;
    m->keys = malloc(cap * m->n_words * sizeof(uint64_t));
    m->values = malloc(cap * sizeof(double));
    if (!m->keys || !m->values) {
        orc_map_free(m);
        return ORC_ENOMEM;
    }
    m->capacity = cap;
    m->len = len;
    if (len) {
        memcpy(m->keys, keys, len * m->n_words * sizeof(uint64_t));
        memcpy(m->values, values, len * sizeof(double));
    }
    return ORC_OK;
}

/*
 * Raw branch of `count` terms into slots 2k, 2k+1 (tpgp_rev.c:432-467; the
 * CUDA ABI's contract is engine/include/tpgp_cuda_rev.h:26-41).  Returns 1
 * for nonzero padding bits and 4 for nonfinite inputs or outputs, as the
 * CUDA branch backend does (engine/src/cuda_rev.cu:88,94,112-113,254-256).
 */
int orc_branches(const uint64_t *keys, const double *values, size_t count, size_t words,
                 size_t spins, size_t i, size_t j, unsigned qi, unsigned qj, double c, double s,
                 double rc, double rs, int enclose, uint64_t *out_keys, double *out_values,
                 double *out_radii) {
    int padding = 0, nonfinite = 0;
    size_t rem = spins % 32;
    for (size_t k = 0; k < count; k++) {
        const uint64_t *key = keys + k * words;
        uint64_t *first = out_keys + 2 * k * words, *second = first + words;
        if (rem && (key[words - 1] >> (2 * rem)))
            padding = 1;
        memcpy(first, key, words * sizeof(uint64_t));
        memcpy(second, key, words * sizeof(uint64_t));
        double v = values[k];
        if (!isfinite(v))
            nonfinite = 1;
        unsigned pi = site_symbol(key, i), pj = site_symbol(key, j);
        out_radii[2 * k] = out_radii[2 * k + 1] = 0;
        if (!(anticommutes(qi, pi) ^ anticommutes(qj, pj))) {
            out_values[2 * k] = v;
            out_values[2 * k + 1] = 0;
            continue;
        }
        unsigned phase = (phase_of(qi, pi) + phase_of(qj, pj)) & 3u;
        second[i / 32] ^= (uint64_t)qi << (2 * (i % 32));
        second[j / 32] ^= (uint64_t)qj << (2 * (j % 32));
        double x = v * c, y = v * s;
        out_values[2 * k] = x;
        out_values[2 * k + 1] = (phase == 1 ? 1.0 : -1.0) * y;
        if (enclose) {
            out_radii[2 * k] = up_add(up_mul(fabs(v), rc), rounding_radius(x));
            out_radii[2 * k + 1] = up_add(up_mul(fabs(v), rs), rounding_radius(y));
        }
        if (!isfinite(x) || !isfinite(y) || !isfinite(out_radii[2 * k]) ||
            !isfinite(out_radii[2 * k + 1]))
            nonfinite = 1;
    }
    return padding ? 1 : nonfinite ? 4 : 0;
}

/* The installed branch backend, if any (tpgp_oracle.h). */
static orc_branch_fn g_branch_fn;
static void *g_branch_user;

void orc_set_branch_backend(orc_branch_fn fn, void *user) {
    g_branch_fn = fn;
    g_branch_user = user;
}

static int size_mul(size_t a, size_t b, size_t *out) {
    if (b && a > SIZE_MAX / b)
        return 0;
    *out = a * b;
    return 1;
}

/*
 * One non-validated rotation exp(-i theta Q) . exp(+i theta Q), theta = h *
 * duration (tpgp_rev.c:535-771 with validated = 0, so every radius is zero
 * and arithmetic_l2 is unchanged).  Transactional: the map and ledger change
 * only on success.  `threads` > 1 splits the branch loop across OpenMP
 * threads, exactly the part the reference parallelises (tpgp_rev.c:641-679).
 */
int orc_rotate(orc_map *map, size_t i, size_t j, unsigned qi, unsigned qj, double h,
               double duration, double threshold, size_t max_terms, double max_drop_l2,
               unsigned threads, orc_ledger *ledger) {
    if (!map || !ledger || !map->n_spins || map->n_words != (map->n_spins + 31) / 32 ||
        i >= map->n_spins || j >= map->n_spins || i == j || qi > 3 || qj > 3 || !isfinite(h) ||
        !isfinite(duration) || !isfinite(threshold) || threshold < 0 || !isfinite(max_drop_l2) ||
        max_drop_l2 < 0 || threads == 0)
        return ORC_EINVAL;
    if (!isfinite(ledger->dropped_l1) || ledger->dropped_l1 < 0 || !isfinite(ledger->dropped_l2) ||
        ledger->dropped_l2 < 0 || !isfinite(ledger->dropped_l2_squared) ||
        ledger->dropped_l2_squared < 0 || !isfinite(ledger->arithmetic_l2) ||
        ledger->arithmetic_l2 < 0)
        return ORC_EINVAL;
    double c, s;
    if (!isfinite(2 * h * duration))
        return ORC_ENUMERIC;
    orc_trig(h, duration, &c, &s);
    if (h == 0 || duration == 0 || map->len == 0)
        return ORC_OK;
    const size_t words = map->n_words, n = map->len;
    if (n > SIZE_MAX / 2)
        return ORC_ENOMEM;
    const size_t slots = 2 * n;
    size_t key_bytes;
    if (!size_mul(slots, words * sizeof(uint64_t), &key_bytes))
        return ORC_ENOMEM;
    uint64_t *raw_keys = malloc(key_bytes), *out_keys = malloc(key_bytes);
    double *raw_values = malloc(slots * sizeof(double)), *out_values = malloc(slots * sizeof(double));
    double *removed = malloc(slots * sizeof(double));
    size_t *idx = malloc(slots * sizeof(size_t)), *tmp = malloc(slots * sizeof(size_t));
    int status = ORC_OK;
    if (!raw_keys || !out_keys || !raw_values || !out_values || !removed || !idx || !tmp) {
        status = ORC_ENOMEM;
        goto out;
    }
    /* branch: from an installed backend (tpgp_rev.c:622-640; its status
     * already mapped to the engine's), else the loop below, the only parallel
     * part, as in the reference */
    if (g_branch_fn) {
        status = g_branch_fn(g_branch_user, map->keys, map->values, n, words, map->n_spins, i, j,
                             qi, qj, c, s, raw_keys, raw_values);
        if (status)
            goto out;
    } else {
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads) schedule(static) if (threads > 1)
#endif
        for (size_t k = 0; k < n; k++) {
            const uint64_t *key = map->keys + k * words;
            uint64_t *first = raw_keys + 2 * k * words, *second = first + words;
            memcpy(first, key, words * sizeof(uint64_t));
            memcpy(second, key, words * sizeof(uint64_t));
            double v = map->values[k];
            unsigned pi = site_symbol(key, i), pj = site_symbol(key, j);
            if (!(anticommutes(qi, pi) ^ anticommutes(qj, pj))) {
                raw_values[2 * k] = v;
                raw_values[2 * k + 1] = 0;
                continue;
            }
            unsigned phase = (phase_of(qi, pi) + phase_of(qj, pj)) & 3u;
            second[i / 32] ^= (uint64_t)qi << (2 * (i % 32));
            second[j / 32] ^= (uint64_t)qj << (2 * (j % 32));
            raw_values[2 * k] = v * c;
            raw_values[2 * k + 1] = (phase == 1 ? 1.0 : -1.0) * (v * s);
        }
    }
    /* finite check (tpgp_rev.c:682-688) */
    for (size_t k = 0; k < slots; k++) {
        if (!isfinite(raw_values[k])) {
            status = ORC_ENUMERIC;
            goto out;
        }
        idx[k] = k;
    }
    /* Stable bottom-up merge sort of slot indices by key.  The reference uses
     * a top-down stable merge sort (tpgp_rev.c:468-483); a stable sort's
     * output permutation is unique, so both give the same order. */
    {
        size_t *a = idx, *b = tmp;
        for (size_t width = 1; width < slots; width *= 2) {
            for (size_t lo = 0; lo < slots; lo += 2 * width) {
                size_t mid = lo + width < slots ? lo + width : slots;
                size_t hi = lo + 2 * width < slots ? lo + 2 * width : slots;
                size_t x = lo, y = mid, o = lo;
                while (x < mid && y < hi) {
                    if (key_order(raw_keys + a[x] * words, raw_keys + a[y] * words, words) <= 0)
                        b[o++] = a[x++];
                    else
                        b[o++] = a[y++];
                }
                while (x < mid)
                    b[o++] = a[x++];
                while (y < hi)
                    b[o++] = a[y++];
            }
            size_t *t = a;
            a = b;
            b = t;
        }
        if (a != idx)
            memcpy(idx, a, slots * sizeof(size_t));
    }
    /* merge duplicates, drop exact zeros, threshold with ledger (tpgp_rev.c:693-729) */
    size_t out_len = 0, discarded = 0;
    double l1 = 0, sq = 0;
    for (size_t k = 0; k < slots;) {
        size_t p = idx[k++];
        const uint64_t *key = raw_keys + p * words;
        double v = raw_values[p];
        while (k < slots && key_order(key, raw_keys + idx[k] * words, words) == 0)
            v += raw_values[idx[k++]];
        if (!isfinite(v)) {
            status = ORC_ENUMERIC;
            goto out;
        }
        if (v == 0)
            continue;
        int identity = 1;
        for (size_t w = 0; w < words; w++)
            identity &= key[w] == 0;
        if (!identity && fabs(v) <= threshold) {
            removed[discarded++] = fabs(v);
            l1 = up_add(l1, fabs(v));
            sq = up_add(sq, up_mul(v, v));
            continue;
        }
        memcpy(out_keys + out_len * words, key, words * sizeof(uint64_t));
        out_values[out_len++] = v;
    }
    /* cap, ledger, budget, commit (tpgp_rev.c:730-757); the removed-L2 bound
     * is the non-MPFR upper_l2 (tpgp_rev.c:58-61) */
    if (max_terms && out_len > max_terms) {
        status = ORC_ECAP;
        goto out;
    }
    {
        double sum = 0;
        for (size_t k = 0; k < discarded; k++)
            sum = up_add(sum, up_mul(removed[k], removed[k]));
        double l2 = sum == 0 ? 0 : nextafter(sqrt(sum), INFINITY);
        orc_ledger next = *ledger;
        next.dropped_l1 = up_add(next.dropped_l1, l1);
        next.dropped_l2 = up_add(next.dropped_l2, l2);
        next.dropped_l2_squared = up_add(next.dropped_l2_squared, sq);
        next.arithmetic_l2 = up_add(next.arithmetic_l2, 0);
        next.rotations++;
        if (discarded)
            next.removal_events++;
        if (out_len > next.peak_terms)
            next.peak_terms = out_len;
        next.arithmetic_enclosed = 0;
        if (!isfinite(next.dropped_l2) || !isfinite(next.arithmetic_l2)) {
            status = ORC_ENUMERIC;
            goto out;
        }
        if (max_drop_l2 && next.dropped_l2 > max_drop_l2) {
            status = ORC_EBUDGET;
            goto out;
        }
        free(map->keys);
        free(map->values);
        map->keys = out_keys;
        map->values = out_values;
        map->len = out_len;
        map->capacity = slots;
        out_keys = NULL;
        out_values = NULL;
        *ledger = next;
    }
out:
    free(raw_keys);
    free(out_keys);
    free(raw_values);
    free(out_values);
    free(removed);
    free(idx);
    free(tmp);
    return status;
}

/*
 * One validated rotation with caller-supplied trigonometric factors c, s and
 * their error radii rc, rs: rotate_product with validated = 1 (tpgp_rev.c:
 * 535-771), where the reference takes c, s, rc, rs from MPFR enclosures
 * (:484-523).  Every raw child carries a radius: 0 for a commuting key's
 * children, upadd(upmul(|v|, rc), round_radius(v c)) and
 * upadd(upmul(|v|, rs), round_radius(v s)) for an anticommuting key's
 * (:459-464); a nonfinite child value or radius is ENUMERIC (:682-688).
 * Merging adds the radii of a key's contributions with upadd, and when two
 * nonzero contributions meet, the rounding radius of their sum (:699-706);
 * every output key with a nonzero merged radius, kept, removed or zero,
 * enters arithmetic_l2's upper L2 in key order (:711-712, :734-738), here
 * the reference's non-MPFR upper_l2 (:57-62).  Keys, values and the dropped
 * sums are those of the non-validated rotation.  An empty map is a no-op.
 */
int orc_rotate_enclosed(orc_map *map, size_t i, size_t j, unsigned qi, unsigned qj, double c,
                        double s, double rc, double rs, double threshold, size_t max_terms,
                        double max_drop_l2, orc_ledger *ledger) {
    if (!map || !ledger || !map->n_spins || map->n_words != (map->n_spins + 31) / 32 ||
        i >= map->n_spins || j >= map->n_spins || i == j || qi > 3 || qj > 3 || !isfinite(c) ||
        !isfinite(s) || !isfinite(rc) || !isfinite(rs) || rc < 0 || rs < 0 ||
        !isfinite(threshold) || threshold < 0 || !isfinite(max_drop_l2) || max_drop_l2 < 0)
        return ORC_EINVAL;
    if (!isfinite(ledger->dropped_l1) || ledger->dropped_l1 < 0 || !isfinite(ledger->dropped_l2) ||
        ledger->dropped_l2 < 0 || !isfinite(ledger->dropped_l2_squared) ||
        ledger->dropped_l2_squared < 0 || !isfinite(ledger->arithmetic_l2) ||
        ledger->arithmetic_l2 < 0)
        return ORC_EINVAL;
    if (map->len == 0)
        return ORC_OK;
    const size_t words = map->n_words, n = map->len, slots = 2 * n;
    uint64_t *raw_keys = malloc(slots * words * sizeof(uint64_t));
    uint64_t *out_keys = malloc(slots * words * sizeof(uint64_t));
    double *raw_values = malloc(slots * sizeof(double)), *out_values = malloc(slots * sizeof(double));
    double *rad = calloc(slots, sizeof(double)), *removed = malloc(slots * sizeof(double));
    double *merged = malloc(slots * sizeof(double));
    size_t *idx = malloc(slots * sizeof(size_t)), *tmp = malloc(slots * sizeof(size_t));
    int status = ORC_OK;
    if (!raw_keys || !out_keys || !raw_values || !out_values || !rad || !removed || !merged ||
        !idx || !tmp) {
        status = ORC_ENOMEM;
        goto out;
    }
    for (size_t k = 0; k < n; k++) {
        const uint64_t *key = map->keys + k * words;
        uint64_t *first = raw_keys + 2 * k * words, *second = first + words;
        memcpy(first, key, words * sizeof(uint64_t));
        memcpy(second, key, words * sizeof(uint64_t));
        double v = map->values[k];
        unsigned pi = site_symbol(key, i), pj = site_symbol(key, j);
        if (!(anticommutes(qi, pi) ^ anticommutes(qj, pj))) {
            raw_values[2 * k] = v;
            raw_values[2 * k + 1] = 0;
            continue;
        }
        unsigned phase = (phase_of(qi, pi) + phase_of(qj, pj)) & 3u;
        second[i / 32] ^= (uint64_t)qi << (2 * (i % 32));
        second[j / 32] ^= (uint64_t)qj << (2 * (j % 32));
        double x = v * c, y = v * s;
        raw_values[2 * k] = x;
        raw_values[2 * k + 1] = (phase == 1 ? 1.0 : -1.0) * y;
        rad[2 * k] = up_add(up_mul(fabs(v), rc), rounding_radius(x));
        rad[2 * k + 1] = up_add(up_mul(fabs(v), rs), rounding_radius(y));
    }
    for (size_t k = 0; k < slots; k++) {
        if (!isfinite(raw_values[k]) || !isfinite(rad[k])) {
            status = ORC_ENUMERIC;
            goto out;
        }
        idx[k] = k;
    }
    {  /* stable bottom-up merge sort of slot indices by key (as orc_rotate) */
        size_t *a = idx, *b = tmp;
        for (size_t width = 1; width < slots; width *= 2) {
            for (size_t lo = 0; lo < slots; lo += 2 * width) {
                size_t mid = lo + width < slots ? lo + width : slots;
                size_t hi = lo + 2 * width < slots ? lo + 2 * width : slots;
                size_t x = lo, y = mid, o = lo;
                while (x < mid && y < hi) {
                    if (key_order(raw_keys + a[x] * words, raw_keys + a[y] * words, words) <= 0)
                        b[o++] = a[x++];
                    else
                        b[o++] = a[y++];
                }
                while (x < mid)
                    b[o++] = a[x++];
                while (y < hi)
                    b[o++] = a[y++];
            }
            size_t *t = a;
            a = b;
            b = t;
        }
        if (a != idx)
            memcpy(idx, a, slots * sizeof(size_t));
    }
    size_t out_len = 0, discarded = 0, nrad = 0;
    double l1 = 0, sq = 0;
    for (size_t k = 0; k < slots;) {
        size_t p = idx[k++];
        const uint64_t *key = raw_keys + p * words;
        double v = raw_values[p], r = rad[p];
        while (k < slots && key_order(key, raw_keys + idx[k] * words, words) == 0) {
            size_t q = idx[k++];
            double previous = v;
            v += raw_values[q];
            r = up_add(r, rad[q]);
            if (previous != 0 && raw_values[q] != 0)
                r = up_add(r, rounding_radius(v));
        }
        if (!isfinite(v) || !isfinite(r)) {
            status = ORC_ENUMERIC;
            goto out;
        }
        if (r != 0)
            merged[nrad++] = r;
        if (v == 0)
            continue;
        int identity = 1;
        for (size_t w = 0; w < words; w++)
            identity &= key[w] == 0;
        if (!identity && fabs(v) <= threshold) {
            removed[discarded++] = fabs(v);
            l1 = up_add(l1, fabs(v));
            sq = up_add(sq, up_mul(v, v));
            continue;
        }
        memcpy(out_keys + out_len * words, key, words * sizeof(uint64_t));
        out_values[out_len++] = v;
    }
    if (max_terms && out_len > max_terms) {
        status = ORC_ECAP;
        goto out;
    }
    {
        double sum = 0, rsum = 0;
        for (size_t k = 0; k < discarded; k++)
            sum = up_add(sum, up_mul(removed[k], removed[k]));
        for (size_t k = 0; k < nrad; k++)
            rsum = up_add(rsum, up_mul(merged[k], merged[k]));
        double l2 = sum == 0 ? 0 : nextafter(sqrt(sum), INFINITY);
        double ar = rsum == 0 ? 0 : nextafter(sqrt(rsum), INFINITY);
        orc_ledger next = *ledger;
        next.dropped_l1 = up_add(next.dropped_l1, l1);
        next.dropped_l2 = up_add(next.dropped_l2, l2);
        next.dropped_l2_squared = up_add(next.dropped_l2_squared, sq);
        next.arithmetic_l2 = up_add(next.arithmetic_l2, ar);
        next.rotations++;
        if (discarded)
            next.removal_events++;
        if (out_len > next.peak_terms)
            next.peak_terms = out_len;
        next.arithmetic_enclosed = 0;  /* no MPFR: tpgp_rev.c:744 */
        if (!isfinite(next.dropped_l2) || !isfinite(next.arithmetic_l2)) {
            status = ORC_ENUMERIC;
            goto out;
        }
        if (max_drop_l2 && next.dropped_l2 > max_drop_l2) {
            status = ORC_EBUDGET;
            goto out;
        }
        free(map->keys);
        free(map->values);
        map->keys = out_keys;
        map->values = out_values;
        map->len = out_len;
        map->capacity = slots;
        out_keys = NULL;
        out_values = NULL;
        *ledger = next;
    }
out:
    free(raw_keys);
    free(out_keys);
    free(raw_values);
    free(out_values);
    free(rad);
    free(removed);
    free(merged);
    free(idx);
    free(tmp);
    return status;
}

/* A list of validated rotations applied in order, transactional over the
 * list (the map and ledger change only when every rotation succeeds). */
typedef struct {
    size_t i, j;
    unsigned qi, qj;
    double c, s, rc, rs;
} orc_rotation;
int orc_rotations_enclosed(orc_map *map, const orc_rotation *rots, size_t count, double threshold,
                           size_t max_terms, double max_drop_l2, orc_ledger *ledger) {
    if (!map || (!rots && count) || !ledger)
        return ORC_EINVAL;
    orc_map work;
    int status = orc_map_from_arrays(&work, map->n_spins, map->keys, map->values, map->len);
    if (status)
        return status;
    orc_ledger next = *ledger;
    for (size_t k = 0; k < count && !status; k++)
        status = orc_rotate_enclosed(&work, rots[k].i, rots[k].j, rots[k].qi, rots[k].qj,
                                     rots[k].c, rots[k].s, rots[k].rc, rots[k].rs, threshold,
                                     max_terms, max_drop_l2, &next);
    if (status) {
        orc_map_free(&work);
        return status;
    }
    orc_map_free(map);
    *map = work;
    *ledger = next;
    return ORC_OK;
}

static int map_copy(orc_map *dst, const orc_map *src) {
    return orc_map_from_arrays(dst, src->n_spins, src->keys, src->values, src->len);
}

/* Symmetric Strang product (tpgp_rev.c:776-809): terms forward at dt/2,
 * then backward at dt/2; transactional over the whole step. */
int orc_strang_step(orc_map *map, const orc_term *terms, size_t count, double dt, double threshold,
                    size_t max_terms, double max_drop_l2, unsigned threads, orc_ledger *ledger) {
    if (!map || (!terms && count) || !ledger || !isfinite(dt))
        return ORC_EINVAL;
    double half = dt * 0.5;
    if (half * 2 != dt)
        return ORC_ENUMERIC;
    orc_map work;
    int status = map_copy(&work, map);
    if (status)
        return status;
    orc_ledger next = *ledger;
    for (size_t k = 0; k < 2 * count && !status; k++) {
        const orc_term *t = k < count ? terms + k : terms + (2 * count - 1 - k);
        status = orc_rotate(&work, t->i, t->j, t->qi, t->qj, t->h, half, threshold, max_terms,
                            max_drop_l2, threads, &next);
    }
    if (status) {
        orc_map_free(&work);
        return status;
    }
    orc_map_free(map);
    *map = work;
    *ledger = next;
    return ORC_OK;
}

/* Adds v into a sorted map the way tpgp_map_add does (tpgp_rev.c:206-243):
 * zero v is ignored; an existing key takes RN(old + v) and disappears when
 * that is zero; a nonfinite sum is ENUMERIC; a new key is inserted in order. */
static int map_add_sorted(orc_map *m, const uint64_t *key, double v) {
    if (!isfinite(v))
        return ORC_EINVAL;
    if (v == 0)
        return ORC_OK;
    const size_t w = m->n_words;
    size_t lo = 0, hi = m->len;
    while (lo < hi) {
        size_t mid = (lo + hi) / 2;
        if (key_order(m->keys + mid * w, key, w) < 0)
            lo = mid + 1;
        else
            hi = mid;
    }
    if (lo < m->len && key_order(m->keys + lo * w, key, w) == 0) {
        double sum = m->values[lo] + v;
        if (!isfinite(sum))
            return ORC_ENUMERIC;
        if (sum == 0) {
            memmove(m->keys + lo * w, m->keys + (lo + 1) * w, (m->len - lo - 1) * w * sizeof(uint64_t));
            memmove(m->values + lo, m->values + lo + 1, (m->len - lo - 1) * sizeof(double));
            m->len--;
        } else {
            m->values[lo] = sum;
        }
        return ORC_OK;
    }
    if (m->len == m->capacity) {
        size_t cap = m->capacity ? 2 * m->capacity : 16;
        uint64_t *k = realloc(m->keys, cap * w * sizeof(uint64_t));
        if (!k)
            return ORC_ENOMEM;
        m->keys = k;
        double *vals = realloc(m->values, cap * sizeof(double));
        if (!vals)
            return ORC_ENOMEM;
        m->values = vals;
        m->capacity = cap;
    }
    memmove(m->keys + (lo + 1) * w, m->keys + lo * w, (m->len - lo) * w * sizeof(uint64_t));
    memmove(m->values + lo + 1, m->values + lo, (m->len - lo) * sizeof(double));
    memcpy(m->keys + lo * w, key, w * sizeof(uint64_t));
    m->values[lo] = v;
    m->len++;
    return ORC_OK;
}

/* The exact algebraic generator -i[H, A] in binary64, no pruning
 * (tpgp_liouvillian, tpgp_rev.c:810-857): for each term in array order (an
 * invalid term is EINVAL when reached), for each input key in key order, an
 * anticommuting key contributes (2h) * v * (+1 if the phase exponent is 1,
 * else -1) to key xor (qi@i, qj@j), added in that order; a nonfinite
 * contribution or sum is ENUMERIC.  `out` is replaced only on success. */
int orc_liouvillian(orc_map *out, const orc_map *in, const orc_term *terms, size_t count) {
    if (!out || !in || (!terms && count))
        return ORC_EINVAL;
    orc_map tmp;
    memset(&tmp, 0, sizeof(tmp));
    tmp.n_spins = in->n_spins;
    tmp.n_words = in->n_words;
    const size_t w = in->n_words;
    uint64_t *key = malloc(w * sizeof(uint64_t));
    if (!key)
        return ORC_ENOMEM;
    int status = ORC_OK;
    for (size_t t = 0; t < count && !status; t++) {
        const orc_term *q = terms + t;
        if (q->i >= in->n_spins || q->j >= in->n_spins || q->i == q->j || q->qi > 3 || q->qj > 3 ||
            !isfinite(q->h)) {
            status = ORC_EINVAL;
            break;
        }
        for (size_t k = 0; k < in->len; k++) {
            const uint64_t *p = in->keys + k * w;
            unsigned pi = site_symbol(p, q->i), pj = site_symbol(p, q->j);
            if (!(anticommutes(q->qi, pi) ^ anticommutes(q->qj, pj)))
                continue;
            unsigned phase = (phase_of(q->qi, pi) + phase_of(q->qj, pj)) & 3u;
            double v = 2 * q->h * in->values[k] * (phase == 1 ? 1 : -1);
            if (!isfinite(v)) {
                status = ORC_ENUMERIC;
                break;
            }
            memcpy(key, p, w * sizeof(uint64_t));
            key[q->i / 32] ^= (uint64_t)q->qi << (2 * (q->i % 32));
            key[q->j / 32] ^= (uint64_t)q->qj << (2 * (q->j % 32));
            status = map_add_sorted(&tmp, key, v);
            if (status)
                break;
        }
    }
    free(key);
    if (status) {
        orc_map_free(&tmp);
        return status;
    }
    if (!tmp.keys) { /* empty result: keep a valid allocation */
        tmp.keys = malloc(w * sizeof(uint64_t));
        tmp.values = malloc(sizeof(double));
        tmp.capacity = 1;
        if (!tmp.keys || !tmp.values) {
            orc_map_free(&tmp);
            return ORC_ENOMEM;
        }
    }
    orc_map_free(out);
    *out = tmp;
    return ORC_OK;
}

/* The same generator for maps too large for sorted insertion: every
 * contribution in the reference's addition order (term, then input key),
 * a stable merge sort by output key, then one sequential RN sum per key in
 * that order, kept when nonzero.  A key's running sum is the one
 * tpgp_map_add keeps (a cancellation to zero removes the key, and the next
 * contribution then starts from it exactly as from zero).  Contributions stop
 * at the first invalid term or nonfinite contribution; a nonfinite sum among
 * those generated precedes the stop, so it is ENUMERIC.  Checked against
 * orc_liouvillian on the reference's golden cases. */
int orc_liouvillian_sorted(orc_map *out, const orc_map *in, const orc_term *terms, size_t count) {
    if (!out || !in || (!terms && count))
        return ORC_EINVAL;
    const size_t w = in->n_words;
    int stop = ORC_OK;
    size_t total = 0, valid = 0;
    for (; valid < count; valid++) {
        const orc_term *q = terms + valid;
        if (q->i >= in->n_spins || q->j >= in->n_spins || q->i == q->j || q->qi > 3 || q->qj > 3 ||
            !isfinite(q->h)) {
            stop = ORC_EINVAL;
            break;
        }
        for (size_t k = 0; k < in->len; k++) {
            const uint64_t *p = in->keys + k * w;
            if (anticommutes(q->qi, site_symbol(p, q->i)) ^ anticommutes(q->qj, site_symbol(p, q->j)))
                total++;
        }
    }
    uint64_t *ck = malloc((total ? total : 1) * w * sizeof(uint64_t));
    double *cv = malloc((total ? total : 1) * sizeof(double));
    size_t *idx = malloc((total ? total : 1) * sizeof(size_t));
    size_t *tmp = malloc((total ? total : 1) * sizeof(size_t));
    int status = ORC_OK;
    if (!ck || !cv || !idx || !tmp) {
        status = ORC_ENOMEM;
        goto done;
    }
    size_t a = 0;
    for (size_t t = 0; t < valid && !status; t++) {
        const orc_term *q = terms + t;
        for (size_t k = 0; k < in->len; k++) {
            const uint64_t *p = in->keys + k * w;
            unsigned pi = site_symbol(p, q->i), pj = site_symbol(p, q->j);
            if (!(anticommutes(q->qi, pi) ^ anticommutes(q->qj, pj)))
                continue;
            unsigned phase = (phase_of(q->qi, pi) + phase_of(q->qj, pj)) & 3u;
            double v = 2 * q->h * in->values[k] * (phase == 1 ? 1 : -1);
            if (!isfinite(v)) {
                status = ORC_ENUMERIC;
                break;
            }
            memcpy(ck + a * w, p, w * sizeof(uint64_t));
            ck[a * w + q->i / 32] ^= (uint64_t)q->qi << (2 * (q->i % 32));
            ck[a * w + q->j / 32] ^= (uint64_t)q->qj << (2 * (q->j % 32));
            cv[a] = v;
            idx[a] = a;
            a++;
        }
    }
    if (status)
        goto done;
    {
        size_t *x0 = idx, *y0 = tmp;
        for (size_t width = 1; width < a; width *= 2) {
            for (size_t lo = 0; lo < a; lo += 2 * width) {
                size_t mid = lo + width < a ? lo + width : a;
                size_t hi = lo + 2 * width < a ? lo + 2 * width : a;
                size_t x = lo, y = mid, o = lo;
                while (x < mid && y < hi) {
                    if (key_order(ck + x0[x] * w, ck + x0[y] * w, w) <= 0)
                        y0[o++] = x0[x++];
                    else
                        y0[o++] = x0[y++];
                }
                while (x < mid)
                    y0[o++] = x0[x++];
                while (y < hi)
                    y0[o++] = x0[y++];
            }
            size_t *t = x0;
            x0 = y0;
            y0 = t;
        }
        if (x0 != idx)
            memcpy(idx, x0, a * sizeof(size_t));
    }
    orc_map res;
    memset(&res, 0, sizeof(res));
    res.n_spins = in->n_spins;
    res.n_words = w;
    res.keys = malloc((a ? a : 1) * w * sizeof(uint64_t));
    res.values = malloc((a ? a : 1) * sizeof(double));
    res.capacity = a ? a : 1;
    if (!res.keys || !res.values) {
        orc_map_free(&res);
        status = ORC_ENOMEM;
        goto done;
    }
    for (size_t k = 0; k < a;) {
        const size_t first = idx[k++];
        double v = cv[first];
        while (k < a && key_order(ck + first * w, ck + idx[k] * w, w) == 0) {
            v += cv[idx[k++]];
            if (!isfinite(v))
                status = ORC_ENUMERIC;
        }
        if (v != 0) {
            memcpy(res.keys + res.len * w, ck + first * w, w * sizeof(uint64_t));
            res.values[res.len++] = v;
        }
    }
    if (!status)
        status = stop;
    if (status) {
        orc_map_free(&res);
    } else {
        orc_map_free(out);
        *out = res;
    }
done:
    free(ck);
    free(cv);
    free(idx);
    free(tmp);
    return status;
}

/* Compensated long-double sum of coefficients whose key has Pauli weight 1
 * with symbol p (tpgp_rev.c:311-338). */
double orc_single_sum(const orc_map *m, unsigned p) {
    if (p < 1 || p > 3)
        return NAN;
    long double sum = 0, correction = 0;
    for (size_t k = 0; k < m->len; k++) {
        unsigned weight = 0, symbol = 0;
        for (size_t w = 0; w < m->n_words; w++) {
            for (uint64_t q = m->keys[k * m->n_words + w]; q; q >>= 2) {
                if (q & 3u) {
                    weight++;
                    symbol = (unsigned)(q & 3u);
                }
            }
        }
        if (weight != 1 || symbol != p)
            continue;
        long double value = m->values[k], next = sum + value;
        if (fabsl(sum) >= fabsl(value))
            correction += (sum - next) + value;
        else
            correction += (value - next) + sum;
        sum = next;
    }
    return (double)(sum + correction);
}

/* Same reduction over caller arrays (used to check the device readout). */
double orc_single_sum_arrays(const uint64_t *keys, const double *values, size_t len,
                             size_t n_spins, unsigned p) {
    orc_map view = {n_spins, (n_spins + 31) / 32, len, len, (uint64_t *)keys, (double *)values};
    return orc_single_sum(&view, p);
}

int orc_has_openmp(void) {
#ifdef _OPENMP
    return 1;
#else
    return 0;
#endif
}
int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---------------------------------------------------------------------------
 * Strang splitting error bound per step (tpgp_rev.c:875-961), the pf term of
 * the CLI's observable bound (cli_rev.c:549-587).  Every sum and product is
 * rounded upward (up_add/up_mul) in the reference's order, so the result is
 * bitwise the reference's.
 *
 * Taylor bound: (2/3) (lambda |dt|)^3 with lambda = sum |h_k| (tpgp_rev.c:875-890).
 * Commutator bound: 2 C |dt|^3 with
 *   C = sum_a [ h_a^2 (sum_{b in N(a), b > a} |h_b|) / 6
 *              + sum_{b in N(a), b > a} |h_a h_b| (sum_{c in N(a) xor N(b), c > a} |h_c|) / 3 ]
 * where N(a) are the terms that anticommute with term a (both h nonzero),
 * ascending; the bound is the smaller of the two (tpgp_rev.c:891-961). */
static int single_anticommutes(unsigned q, unsigned p) { return q && p && q != p; }

static int terms_anticommute(const orc_term *a, const orc_term *b) {
    int odd = 0;
    if (a->i == b->i) odd ^= single_anticommutes(a->qi, b->qi);
    if (a->i == b->j) odd ^= single_anticommutes(a->qi, b->qj);
    if (a->j == b->i) odd ^= single_anticommutes(a->qj, b->qi);
    if (a->j == b->j) odd ^= single_anticommutes(a->qj, b->qj);
    return odd;
}

double orc_strang_bound_taylor(const orc_term *terms, size_t count, double dt) {
    if ((!terms && count) || !isfinite(dt))
        return NAN;
    double lambda = 0;
    for (size_t k = 0; k < count; k++) {
        const orc_term *t = terms + k;
        if (!isfinite(t->h) || t->i == t->j || t->qi > 3 || t->qj > 3)
            return NAN;
        lambda = up_add(lambda, fabs(t->h));
    }
    const double x = up_mul(lambda, fabs(dt));
    return up_mul(up_mul(up_mul(x, x), x), nextafter(2.0 / 3.0, INFINITY));
}

double orc_strang_bound(const orc_term *terms, size_t count, double dt) {
    const double taylor = orc_strang_bound_taylor(terms, count, dt);
    if (isnan(taylor))
        return NAN;
    /* anticommutation graph as a CSR structure, rows ascending */
    size_t *degree = calloc(count + 1, sizeof(size_t));
    if (!degree)
        return taylor;
    for (size_t a = 0; a < count; a++)
        for (size_t b = a + 1; b < count; b++)
            if (terms[a].h != 0 && terms[b].h != 0 && terms_anticommute(terms + a, terms + b)) {
                degree[a]++;
                degree[b]++;
            }
    size_t *start = malloc((count + 1) * sizeof(size_t));
    size_t total = 0;
    for (size_t a = 0; a < count; a++)
        total += degree[a];
    size_t *adj = malloc((total ? total : 1) * sizeof(size_t));
    size_t *fill = calloc(count + 1, sizeof(size_t));
    if (!start || !adj || !fill) {
        free(degree);
        free(start);
        free(adj);
        free(fill);
        return taylor;
    }
    start[0] = 0;
    for (size_t a = 0; a < count; a++)
        start[a + 1] = start[a] + degree[a];
    /* pairs in (a ascending, b ascending) order keep every row sorted */
    for (size_t a = 0; a < count; a++)
        for (size_t b = a + 1; b < count; b++)
            if (terms[a].h != 0 && terms[b].h != 0 && terms_anticommute(terms + a, terms + b)) {
                adj[start[a] + fill[a]++] = b;
                adj[start[b] + fill[b]++] = a;
            }
    const double sixth = nextafter(1.0 / 6.0, INFINITY), third = nextafter(1.0 / 3.0, INFINITY);
    double C = 0;
    for (size_t a = 0; a < count; a++) {
        const double ha = fabs(terms[a].h);
        const size_t *na = adj + start[a];
        const size_t da = degree[a];
        double later = 0;
        for (size_t k = 0; k < da; k++)
            if (na[k] > a)
                later = up_add(later, fabs(terms[na[k]].h));
        C = up_add(C, up_mul(up_mul(up_mul(ha, ha), later), sixth));
        for (size_t k = 0; k < da; k++) {
            const size_t b = na[k];
            if (b <= a)
                continue;
            const size_t *nb = adj + start[b];
            const size_t db = degree[b];
            size_t x = 0, y = 0;
            double odd = 0;
            /* ascending walk over N(a) xor N(b) */
            while (x < da || y < db) {
                size_t c;
                if (y == db || (x < da && na[x] < nb[y])) {
                    c = na[x++];
                } else if (x == da || nb[y] < na[x]) {
                    c = nb[y++];
                } else {
                    x++;
                    y++;
                    continue;
                }
                if (c > a)
                    odd = up_add(odd, fabs(terms[c].h));
            }
            C = up_add(C, up_mul(up_mul(up_mul(ha, fabs(terms[b].h)), odd), third));
        }
    }
    free(degree);
    free(start);
    free(adj);
    free(fill);
    const double t = fabs(dt);
    const double nested = up_mul(up_mul(up_mul(up_mul(2, C), t), t), t);
    return fmin(taylor, nested);
}
