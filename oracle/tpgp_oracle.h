/*
 * CPU oracle for the Pauli-propagation branch step: types and entry points.
 *
 * TEST INFRASTRUCTURE ONLY (see tpgp_oracle.c).  C test programs include this
 * header and link oracle/_build/liborc.so; the Python side binds the same
 * layouts through ctypes (oracle/oracle.py).  No product code includes it.
 */
#ifndef TPGP_ORACLE_H
#define TPGP_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes follow tpgp_status (DDevol engine/include/tpgp_rev.h:9-17). */
enum { ORC_OK = 0, ORC_EINVAL, ORC_ENOMEM, ORC_ECAP, ORC_ENUMERIC, ORC_EBACKEND, ORC_EBUDGET };

/* Same field order as tpgp_map / tpgp_ledger / tpgp_term (tpgp_rev.h:25-51). */
typedef struct {
    size_t n_spins, n_words, len, capacity;
    uint64_t *keys;
    double *values;
} orc_map;
typedef struct {
    size_t i, j;
    unsigned qi, qj;
    double h;
    size_t layer;
} orc_term;
typedef struct {
    double dropped_l1, dropped_l2, dropped_l2_squared;
    double arithmetic_l2;
    size_t rotations, removal_events, peak_terms;
    int arithmetic_enclosed;
} orc_ledger;

void orc_trig(double h, double duration, double *c, double *s);
void orc_map_free(orc_map *m);
int orc_map_from_arrays(orc_map *m, size_t n_spins, const uint64_t *keys, const double *values,
                        size_t len);
int orc_branches(const uint64_t *keys, const double *values, size_t count, size_t words,
                 size_t spins, size_t i, size_t j, unsigned qi, unsigned qj, double c, double s,
                 double rc, double rs, int enclose, uint64_t *out_keys, double *out_values,
                 double *out_radii);
int orc_rotate(orc_map *map, size_t i, size_t j, unsigned qi, unsigned qj, double h,
               double duration, double threshold, size_t max_terms, double max_drop_l2,
               unsigned threads, orc_ledger *ledger);
int orc_strang_step(orc_map *map, const orc_term *terms, size_t count, double dt, double threshold,
                    size_t max_terms, double max_drop_l2, unsigned threads, orc_ledger *ledger);
double orc_single_sum(const orc_map *m, unsigned p);

/* A branch backend: writes the 2*count raw children of one non-validated
 * rotation (slots 2k, 2k+1 as orc_branches does) and returns an ORC status.
 * Installed with orc_set_branch_backend, it replaces orc_rotate's own branch
 * loop, the way the reference engine takes the children from its CUDA
 * backend (engine/src/tpgp_rev.c:622-640): the sort, merge, threshold and
 * ledger stay on the host.  NULL restores the built-in loop.  Process-wide;
 * a test sets it before a trajectory and clears it after. */
typedef int (*orc_branch_fn)(void *user, const uint64_t *keys, const double *values, size_t count,
                             size_t words, size_t spins, size_t i, size_t j, unsigned qi,
                             unsigned qj, double c, double s, uint64_t *out_keys,
                             double *out_values);
void orc_set_branch_backend(orc_branch_fn fn, void *user);

#ifdef __cplusplus
}
#endif
#endif
