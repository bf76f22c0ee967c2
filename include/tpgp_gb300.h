/* Device-resident Pauli propagation on one GB300 (sm_103a).
 *
 * The reference engine keeps its operator as a host tpgp_map and, with the
 * CUDA backend, ships every rotation's input to the GPU and its 2n raw
 * children back for a host sort (DDevol engine/src/tpgp_rev.c:622-640,
 * engine/src/cuda_rev.cu:229-264).  This interface keeps the map on the
 * device for the whole rotation: branch, sort by key, merge of duplicates,
 * threshold truncation and ledger all run as sm_103a kernels, and the map
 * crosses PCIe/C2C only on upload and download.  The host map format
 * (keys[k*n_words + w], two bits per site, strictly ascending keys, no zeros)
 * is the reference's tpgp_map, so maps move to and from the reference
 * engine, its checkpoint code and its readout unchanged.
 *
 * Each entry point cites the reference interface it stands in for.  Status
 * codes are tpgp_status's (engine/include/tpgp_rev.h:9-17); every mutation
 * is transactional: on failure the map and the ledger are unchanged.
 */
#ifndef TPGP_GB300_H
#define TPGP_GB300_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Same values as tpgp_status (engine/include/tpgp_rev.h:9-17). */
typedef enum {
    TPGP_GB_OK = 0,
    TPGP_GB_EINVAL,
    TPGP_GB_ENOMEM,
    TPGP_GB_ECAP,
    TPGP_GB_ENUMERIC,
    TPGP_GB_EBACKEND,
    TPGP_GB_EBUDGET
} tpgp_gb_status;

/* Same layout as tpgp_term (engine/include/tpgp_rev.h:30-35). */
typedef struct {
    size_t i, j;
    unsigned qi, qj;
    double h;
    size_t layer;
} tpgp_gb_term;

/* Same layout as tpgp_ledger (engine/include/tpgp_rev.h:46-51). */
typedef struct {
    double dropped_l1, dropped_l2, dropped_l2_squared;
    double arithmetic_l2;
    size_t rotations, removal_events, peak_terms;
    int arithmetic_enclosed;
} tpgp_gb_ledger;

/* Rotation options; threshold, max_terms and max_drop_l2 mean what they mean
 * in tpgp_options (engine/include/tpgp_rev.h:36-45).
 *   exact_ledger = 1: the removed-weight sums are accumulated in the
 *     reference's sequential key order, so the ledger is bitwise equal to the
 *     CPU engine's: each rotation's removed terms are logged, sorted by key
 *     and summed after the step's rotations with warp-parallel upward sums
 *     that give the sequential chain's bits.
 *   exact_ledger = 0: each removed |v| and v^2 is rounded up to a multiple
 *     of a fixed-point unit set by the threshold and summed exactly in 128-bit
 *     integers, then converted up once per rotation: deterministic,
 *     independent of the launch shape, a rigorous upper bound on the removed
 *     weight a few ulps from the sequential sum.  Keys, values, FIDs and the
 *     integer ledger fields are the same in both modes.
 *   With either ledger, steps of maps up to 6e5 terms run the hash-table step
 *   (one kernel per rotation, no sort; TPGP_GB_HASH=0 disables it) and larger
 *   maps the sorted per-rotation kernels.
 *   use_graphs = 1: each Strang step's kernel sequence is captured once as a
 *     CUDA graph and replayed.
 *   wait_polls: how many times a device-side wait (decoupled look-back,
 *     grid barrier) polls before it gives up and the call returns EBACKEND
 *     with the map unchanged; 0 selects the defaults (2^22 look-back polls,
 *     2^24 barrier polls of ~32 ns, far beyond any wait of a healthy run). */
typedef struct {
    double threshold;
    size_t max_terms;
    double max_drop_l2;
    int exact_ledger;
    int use_graphs;
    unsigned wait_polls;
} tpgp_gb_options;

typedef struct tpgp_gb_context tpgp_gb_context;
typedef struct tpgp_gb_map tpgp_gb_map;

/* Library and device.  compiled() returns 1 (the library has its device
 * code).  create() binds one device (index as CUDA_VISIBLE_DEVICES numbers
 * it) and a stream; NULL with a message when the device is missing.  Replaces the context part of
 * engine/include/tpgp_cuda_rev.h:20-23 for the device-resident path. */
int tpgp_gb_compiled(void);
tpgp_gb_options tpgp_gb_default_options(void);
tpgp_gb_context *tpgp_gb_create(int device_index, char *error, size_t error_capacity);
void tpgp_gb_destroy(tpgp_gb_context *context);
const char *tpgp_gb_device_name(const tpgp_gb_context *context);

/* Device maps.  Stand-ins for tpgp_map_init / tpgp_map_free / the map's
 * storage (engine/include/tpgp_rev.h:25-29, 60-61).  n_spins >= 2 and at
 * most 128 (keys of up to four 64-bit words). */
tpgp_gb_status tpgp_gb_map_create(tpgp_gb_context *context, size_t n_spins, tpgp_gb_map **map,
                                  char *error, size_t error_capacity);
void tpgp_gb_map_destroy(tpgp_gb_map *map);
size_t tpgp_gb_map_len(const tpgp_gb_map *map);
size_t tpgp_gb_map_spins(const tpgp_gb_map *map);

/* Replaces the map's contents with `len` host terms.  The terms must satisfy
 * the tpgp_map invariants the reference's tpgp_map_add enforces
 * (engine/src/tpgp_rev.c:73-83, 206-210): keys strictly ascending, zero
 * padding bits, finite nonzero values.  EINVAL otherwise (map unchanged). */
tpgp_gb_status tpgp_gb_map_upload(tpgp_gb_map *map, const uint64_t *keys, const double *values,
                                  size_t len, char *error, size_t error_capacity);

/* Copies the map to host arrays of room for `capacity` terms; *len receives
 * the term count.  EINVAL (nothing copied) if capacity < len. */
tpgp_gb_status tpgp_gb_map_download(const tpgp_gb_map *map, uint64_t *keys, double *values,
                                    size_t capacity, size_t *len, char *error,
                                    size_t error_capacity);

/* One rotation exp(-i theta Q) A exp(+i theta Q), Q = sigma^qi_i sigma^qj_j.
 * Same contract as tpgp_rotate (engine/include/tpgp_rev.h:84-85,
 * engine/src/tpgp_rev.c:772-775) with the non-validated backend: keys,
 * values, cap, budget and statuses are the reference's. */
tpgp_gb_status tpgp_gb_rotate(tpgp_gb_map *map, size_t i, size_t j, unsigned qi, unsigned qj,
                              double theta, const tpgp_gb_options *options,
                              tpgp_gb_ledger *ledger, char *error, size_t error_capacity);

/* Symmetric Strang step: terms forward at dt/2, then backward at dt/2.
 * Same contract as tpgp_strang_step (engine/include/tpgp_rev.h:86-87,
 * engine/src/tpgp_rev.c:776-809). */
tpgp_gb_status tpgp_gb_strang_step(tpgp_gb_map *map, const tpgp_gb_term *terms, size_t count,
                                   double dt, const tpgp_gb_options *options,
                                   tpgp_gb_ledger *ledger, char *error, size_t error_capacity);

/* The step engine's launch configuration for a map.  hash_step: 1 lets
 * steps of maps up to the size crossover run as the hash-table step, 0 keeps
 * every step on the sorted per-rotation kernels; hash_ctas: CTAs per SM of
 * the hash pass (1-4, the pass's grid); hash_pdl / sorted_pdl: programmatic
 * dependent launch between consecutive passes / sorted kernels; hash_fuse:
 * consecutive rotations on one site pair in one fused pass (bound ledger).
 * Results are bitwise the same under every configuration; only the time
 * differs.  step_ms: a measured step time, 0 when not measured. */
typedef struct {
    int hash_step, hash_ctas, hash_pdl, hash_fuse, sorted_pdl;
    double step_ms;
} tpgp_gb_engine_config;

#define TPGP_GB_TUNING_MAX 16
typedef struct {
    tpgp_gb_engine_config chosen;  /* applied to the map */
    tpgp_gb_engine_config before;  /* the map's configuration on entry, timed */
    size_t tried_count;
    tpgp_gb_engine_config tried[TPGP_GB_TUNING_MAX];
} tpgp_gb_tuning;

tpgp_gb_status tpgp_gb_map_get_config(const tpgp_gb_map *map, tpgp_gb_engine_config *config);
tpgp_gb_status tpgp_gb_map_set_config(tpgp_gb_map *map, const tpgp_gb_engine_config *config);

/* Times one Strang step of the terms from the map's current state under
 * each candidate configuration (the engine choice, the hash pass's CTAs per
 * SM, dependent launch, fusion), each after one untimed step that captures
 * its graphs, restoring the state after every trial; applies the fastest and
 * reports all.  The map's contents are unchanged.  Device time by CUDA
 * events, as tpgp_gb_last_elapsed_ms. */
tpgp_gb_status tpgp_gb_map_autotune(tpgp_gb_map *map, const tpgp_gb_term *terms, size_t count,
                                    double dt, const tpgp_gb_options *options,
                                    tpgp_gb_tuning *tuning, char *error, size_t error_capacity);

/* One rotation with the caller's trigonometric factors: c, s the cosine and
 * sine of the angle 2*h*duration, rc, rs >= 0 bounds on their errors (the
 * reference computes these with MPFR, engine/src/tpgp_rev.c:484-523). */
typedef struct {
    size_t i, j;
    unsigned qi, qj;
    double c, s, rc, rs;
} tpgp_gb_rotation;

/* Validated rotations (tpgp_options.validated = 1 in the reference,
 * rotate_product at engine/src/tpgp_rev.c:535-771) with host-supplied
 * factors and radii, in order, transactional over the list.  Keys, values
 * and the dropped sums are those of the plain rotation; every child also
 * carries an error radius, upadd(upmul(|v|, rc), round_radius(v c)) for the
 * cosine child and the same with rs for the sine child (:459-464); merging
 * adds a key's radii and, where two nonzero contributions meet, the
 * rounding radius of their sum (:699-706); and arithmetic_l2 grows by the
 * upper L2 of the nonzero merged radii in key order (:711-712, :734-738;
 * the sum of upmul squares and the next double above its square root, the
 * reference's upper_l2 without MPFR, :57-62).  A nonfinite child or merged
 * radius is ENUMERIC; arithmetic_enclosed becomes 0 (no MPFR enclosure).
 * The ledger is the exact one whatever options.exact_ledger says.  Runs on
 * the hash-table step at any map size.  A list with an invalid rotation
 * (site, generator, or a nonfinite or negative factor or radius) returns
 * EINVAL after the rotations before it are computed, with the map and
 * ledger unchanged (their statuses come first, as in the reference's
 * order); an empty map is a no-op. */
tpgp_gb_status tpgp_gb_rotate_enclosed(tpgp_gb_map *map, const tpgp_gb_rotation *rotations,
                                       size_t count, const tpgp_gb_options *options,
                                       tpgp_gb_ledger *ledger, char *error, size_t error_capacity);

/* `steps` Strang steps in a row, the reference CLI's time loop
 * (engine/src/cli_rev.c:575-670) without I/O: after each accepted step k
 * (0-based) fid_sums[k] receives tpgp_gb_single_sum(map, 1) when fid_sums
 * is not NULL.  *steps_done receives the number of accepted steps; on a
 * failure the map and ledger hold the last accepted step. */
tpgp_gb_status tpgp_gb_evolve(tpgp_gb_map *map, const tpgp_gb_term *terms, size_t count,
                              double dt, size_t steps, const tpgp_gb_options *options,
                              tpgp_gb_ledger *ledger, double *fid_sums, size_t *steps_done,
                              char *error, size_t error_capacity);

/* A restart record in the reference's version-2 checkpoint format
 * (engine/include/checkpoint_rev.h:6-22, engine/src/checkpoint_rev.c:283-387
 * save, :412-586 load): little-endian fields, the terms, the map in key
 * order, and the SHA-256 of that payload; written through a temporary file,
 * fsync and rename, with a .manifest.json beside it.  Host arrays; a record
 * written here loads in the reference engine and the other way round.
 * Zero-initialise before load; release with tpgp_gb_checkpoint_free. */
typedef struct {
    size_t n_spins, len;
    uint64_t *keys;  /* keys[k * ceil(n_spins / 32) + w] */
    double *values;
    tpgp_gb_term *terms;
    size_t term_count;
    double threshold;      /* options: threshold, max_terms, threads, backend, */
    size_t max_terms;      /* validated, max_drop_l2 (tpgp_options fields)     */
    unsigned threads;
    int backend, validated;
    double max_drop_l2;
    tpgp_gb_ledger ledger;
    double dt, pf_bound, residual_bound, max_fid_bound;
    size_t step, total_steps;
    int residual_depth; /* -1: none (residual_bound is then NaN) */
    int initial_global;
    char model[32];
    double j2;
    size_t linear_size, resumed_from_step, prior_total_steps, prior_max_terms;
    int stop_reason; /* 0 running, 1 complete, 2 walltime, 3 signal, 4 resource,
                        5 numerical, 6 accuracy */
    tpgp_gb_status last_status;
} tpgp_gb_checkpoint;

/* Writes a host record (validated as the reference validates one). */
tpgp_gb_status tpgp_gb_checkpoint_write(const char *path, const tpgp_gb_checkpoint *record,
                                        char *error, size_t error_capacity);
/* Reads and validates a record (checksum first); *record is replaced only on
 * success. */
tpgp_gb_status tpgp_gb_checkpoint_load(const char *path, tpgp_gb_checkpoint *record, char *error,
                                       size_t error_capacity);
void tpgp_gb_checkpoint_free(tpgp_gb_checkpoint *record);
/* Downloads a device map and writes it with its run state as the reference
 * CLI's save_current does (engine/src/cli_rev.c:72-106): backend 4 (CUDA),
 * one thread, no validated mode, no residual bound, linear size the cubic
 * model's lattice edge (else 3, the reference CLI's default). */
tpgp_gb_status tpgp_gb_checkpoint_save(const char *path, const tpgp_gb_map *map,
                                       const tpgp_gb_term *terms, size_t count, const char *model,
                                       double j2, double dt, const tpgp_gb_options *options,
                                       const tpgp_gb_ledger *ledger, double pf_bound, size_t step,
                                       size_t total_steps, int initial_global, int stop_reason,
                                       char *error, size_t error_capacity);

/* Hilbert-Schmidt norm of the map's coefficients, sqrt(sum v^2): a
 * deterministic device reduction in binary64 (pairs of doubles carry the
 * sum's rounding error), within a few ulps of tpgp_map_l2's long-double sum
 * (engine/include/tpgp_rev.h:75, engine/src/tpgp_rev.c:266-271). */
tpgp_gb_status tpgp_gb_map_l2(const tpgp_gb_map *map, double *l2);

/* Upward sums of consecutive chains of `chain` addends (the last one may be
 * shorter): out[c] = upadd(...upadd(upadd(0, x[c*chain]), x[c*chain+1])...),
 * upadd(a, b) = nextafter(a + b, +inf) with a zero operand returning the
 * other (engine/src/tpgp_rev.c:25-36), bit for bit the sequential chain;
 * addends >= 0.  The device kernel behind the exact ledger's per-rotation
 * sums and the step's ledger commit, computed by a warp 32 addends at a time.
 * out holds ceil(n / chain) values. */
tpgp_gb_status tpgp_gb_upward_sums(tpgp_gb_context *context, const double *x, size_t n,
                                   size_t chain, double *out);

/* Conservative third-order Strang bound per step for the ordered terms,
 * bitwise equal to tpgp_strang_bound (engine/include/tpgp_rev.h:91-94,
 * engine/src/tpgp_rev.c:887-961); NaN for an invalid term list.  Host
 * arithmetic only. */
double tpgp_gb_strang_bound(const tpgp_gb_term *terms, size_t count, double dt);

/* The exact algebraic generator: *out = -i[H, in] with H = sum of the terms,
 * in binary64 with no pruning, bitwise equal to tpgp_liouvillian
 * (engine/include/tpgp_rev.h:88-90, engine/src/tpgp_rev.c:810-857).  Both
 * maps live on the device, belong to one context and have the same spin
 * count; out may be in.  EINVAL for an invalid term (when no earlier term
 * produced a nonfinite contribution or sum, which is ENUMERIC).  out is
 * unchanged on failure; in is never changed unless it is out. */
tpgp_gb_status tpgp_gb_liouvillian(tpgp_gb_map *out, const tpgp_gb_map *in,
                                   const tpgp_gb_term *terms, size_t count, char *error,
                                   size_t error_capacity);

/* Compensated sum of the coefficients whose key has Pauli weight one with
 * symbol `pauli` (1..3), bitwise equal to tpgp_map_single_sum
 * (engine/include/tpgp_rev.h:73, engine/src/tpgp_rev.c:311-338). */
tpgp_gb_status tpgp_gb_single_sum(const tpgp_gb_map *map, unsigned pauli, double *sum);

/* Measurement of the most recent tpgp_gb_rotate / tpgp_gb_strang_step /
 * tpgp_gb_evolve call (no reference counterpart; the reference CLI records
 * only wall seconds, engine/src/cli_rev.c:572-608):
 *   last_elapsed_ms: device time (CUDA events on the map's stream) from the
 *     call's first launch to its last completion, host gaps included;
 *   last_launches:   kernels launched by the call;
 *   last_terms:      input terms summed over the call's committed rotations
 *                    (the Pauli terms/s numerator). */
double tpgp_gb_last_elapsed_ms(const tpgp_gb_map *map);
size_t tpgp_gb_last_launches(const tpgp_gb_map *map);
size_t tpgp_gb_last_terms(const tpgp_gb_map *map);

/* Per-kernel profile (no reference counterpart).  With profiling on, the
 * next calls launch without graphs and bracket the kernels with CUDA events;
 * kernel_profile then fills TPGP_GB_PROFILE_SLOTS entries with the summed
 * device milliseconds and launch counts since profiling was switched on:
 * sorted path 0 classify, 1 flip-sort, 2 partition, 3 merge (each kernel
 * bracketed); hash-table path 4 rotations, 5 table build, 6 commit chain and
 * extraction, 7 radix sort, 8 stat reduction and the exact ledger's segment
 * sort and sums (bracketed as groups). */
#define TPGP_GB_PROFILE_SLOTS 9
void tpgp_gb_set_profiling(tpgp_gb_map *map, int on);
void tpgp_gb_kernel_profile(const tpgp_gb_map *map, double *milliseconds, size_t *launches);

/* Batched maps (no reference counterpart; the reference runs independent
 * solves as separate processes, scripts/campaign.sh).  A batch holds
 * n_items independent maps (powder orientations, disorder realizations,
 * served requests), each with its own spins, terms, dt and options, and
 * advances all of them by one clustered launch per Strang step, key width and
 * cluster size: every item is owned by one thread-block cluster of G CTAs
 * that runs the item's whole rotation list, and the step's transfers and
 * launches are replayed from a CUDA graph.  G grows with the item's map (one
 * CTA per 8192 terms by default, a power of two from the width's base size up
 * to 16 where the device runs 16-CTA clusters, else 8).  Bound-ledger items
 * whose step fits a CTA-local hash table run there instead, one CTA per
 * item (TPGP_GB_BATCH_SMEM=0 keeps every item on the clusters).  Results per
 * item are those of tpgp_gb_strang_step on that item alone (keys, values,
 * FID bitwise).
 * Items fail independently: item_status() is the tpgp_status of an item's
 * failed step (the item then stays at its last accepted step and is
 * skipped), 0 while healthy. */
typedef struct tpgp_gb_batch tpgp_gb_batch;
tpgp_gb_status tpgp_gb_batch_create(tpgp_gb_context *context, size_t n_items,
                                    const size_t *n_spins, tpgp_gb_batch **batch, char *error,
                                    size_t error_capacity);
void tpgp_gb_batch_destroy(tpgp_gb_batch *batch);
tpgp_gb_status tpgp_gb_batch_upload(tpgp_gb_batch *batch, size_t item, const uint64_t *keys,
                                    const double *values, size_t len, char *error,
                                    size_t error_capacity);
/* The item's Hamiltonian terms, time step and options (as tpgp_gb_strang_step). */
tpgp_gb_status tpgp_gb_batch_set_terms(tpgp_gb_batch *batch, size_t item,
                                       const tpgp_gb_term *terms, size_t count, double dt,
                                       const tpgp_gb_options *options, char *error,
                                       size_t error_capacity);
/* `steps` Strang steps of every healthy item; fid_sums (steps x n_items, may
 * be NULL) receives each item's single_sum(X) after each step (NaN for a
 * failed item and for an idle item: one with no terms or an empty map).
 * Returns a non-OK status only for a device failure. */
tpgp_gb_status tpgp_gb_batch_step(tpgp_gb_batch *batch, size_t steps, double *fid_sums,
                                  char *error, size_t error_capacity);
/* Picks, per key width, from the fastest trial step on the current maps
 * (trial steps are not committed): the base cluster size G in {1, 2, 4, 8};
 * the terms per CTA of the cluster-size rule in {4096, 8192, 16384} (16, 32
 * or 64 terms per thread); whether bound-ledger items that fit run in
 * CTA-local hash tables or on the clusters; and the tables' size, 2 or 4
 * slots per expected claimed key (the table is also the tile of the item's
 * closing block sort).  Results are the same under every choice.
 * tpgp_gb_batch_cluster returns the base size, tpgp_gb_batch_uses_tables 1
 * when the tables are in use, tpgp_gb_batch_get_tuning all of a width's
 * choices (NULL outputs are skipped). */
tpgp_gb_status tpgp_gb_batch_autotune(tpgp_gb_batch *batch, char *error, size_t error_capacity);
int tpgp_gb_batch_cluster(const tpgp_gb_batch *batch, size_t n_words);
int tpgp_gb_batch_uses_tables(const tpgp_gb_batch *batch);
tpgp_gb_status tpgp_gb_batch_get_tuning(const tpgp_gb_batch *batch, size_t n_words, int *cluster,
                                        size_t *terms_per_cta, double *table_slots_per_claim);
/* Sets the base cluster size (a power of two up to max_cluster) and the
 * terms per CTA of the size rule (0: 8192) for one key width. */
tpgp_gb_status tpgp_gb_batch_set_cluster(tpgp_gb_batch *batch, size_t n_words, int base,
                                         size_t terms_per_cta, char *error,
                                         size_t error_capacity);
/* Largest cluster size the device runs for this key width (8 or 16). */
int tpgp_gb_batch_max_cluster(const tpgp_gb_batch *batch, size_t n_words);
int tpgp_gb_batch_item_status(const tpgp_gb_batch *batch, size_t item);
size_t tpgp_gb_batch_len(const tpgp_gb_batch *batch, size_t item);
tpgp_gb_status tpgp_gb_batch_ledger(const tpgp_gb_batch *batch, size_t item,
                                    tpgp_gb_ledger *ledger);
tpgp_gb_status tpgp_gb_batch_download(const tpgp_gb_batch *batch, size_t item, uint64_t *keys,
                                      double *values, size_t capacity, size_t *len, char *error,
                                      size_t error_capacity);
/* Device time (ms), input terms and launches of the last batch_step call. */
double tpgp_gb_batch_last_elapsed_ms(const tpgp_gb_batch *batch);
size_t tpgp_gb_batch_last_terms(const tpgp_gb_batch *batch);
size_t tpgp_gb_batch_last_launches(const tpgp_gb_batch *batch);

/* Serving (no reference counterpart).  A stream of FID solves served with
 * continuous batching: requests are admitted, in arrival order, as soon as
 * they have arrived, a slot of a large enough key width is free and the
 * projected map memory of all admitted solves stays within memory_budget
 * bytes (projection: the mean peak map size seen so far for that key width,
 * 10^4 terms before any solve finished, times the arena bytes per term).
 * Every tick advances all admitted solves by one Strang step in one batched
 * launch; a solve leaves its slot after its last step and a waiting request
 * takes it on the next tick.  Arrival times are seconds after the call
 * starts (wall clock).  fids, when not NULL, receives each request's FID
 * sums after each of its steps, requests concatenated in order.  Each
 * solve's results are those of tpgp_gb_evolve on that request alone with
 * n_spins rounded up to its slot's width (32, 64 or 96 spins). */
typedef struct {
    double arrival;
    size_t n_spins;
    const tpgp_gb_term *terms;
    size_t count;
    double dt;
    size_t steps;
    tpgp_gb_options options;
    const uint64_t *keys; /* initial operator, n_spins-wide keys */
    const double *values;
    size_t len;
} tpgp_gb_request;
typedef struct {
    double admitted, finished; /* seconds after the call started */
    int status;                /* tpgp_status of the solve */
    size_t slot, slot_spins, peak_terms;
    double fid_last;
} tpgp_gb_response;
typedef struct {
    double busy_seconds;      /* device time of all ticks */
    double wall_seconds;      /* wall time of the call */
    unsigned long long ticks; /* batched Strang steps */
    unsigned long long terms; /* input terms summed over all rotations */
    unsigned long long launches;
    size_t max_active;        /* most solves admitted at once */
} tpgp_gb_serve_stats;
/* slots[w] = slots of key width w+1 words (w = 0, 1, 2: up to 32, 64, 96
 * spins).  stats may be NULL. */
tpgp_gb_status tpgp_gb_serve(tpgp_gb_context *context, const tpgp_gb_request *requests,
                             size_t n_requests, const size_t slots[3], size_t memory_budget,
                             double *fids, tpgp_gb_response *responses,
                             tpgp_gb_serve_stats *stats, char *error, size_t error_capacity);

#ifdef __cplusplus
}
#endif
#endif
