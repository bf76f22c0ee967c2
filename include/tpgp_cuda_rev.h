/* Branch-backend C ABI of the GB300 library, byte-compatible with DDevol's
 * CUDA branch backend.  Link libtpgp_gb300.so in place of the reference's
 * engine/src/cuda_rev.cu (or its stub engine/cuda/stub_rev.c) and the engine's
 * TPGP_CUDA backend (engine/src/tpgp_rev.c:622-640) runs on these entry
 * points unchanged.
 *
 * Declarations replace, one for one, DDevol engine/include/tpgp_cuda_rev.h:
 *   tpgp_cuda_context     -> tpgp_cuda_rev.h:9
 *   tpgp_cuda_status      -> tpgp_cuda_rev.h:10-16
 *   tpgp_cuda_compiled    -> tpgp_cuda_rev.h:20
 *   tpgp_cuda_create      -> tpgp_cuda_rev.h:21
 *   tpgp_cuda_destroy     -> tpgp_cuda_rev.h:22
 *   tpgp_cuda_device_name -> tpgp_cuda_rev.h:23
 *   tpgp_cuda_branches    -> tpgp_cuda_rev.h:42-48
 */
#ifndef TPGP_CUDA_REV_H
#define TPGP_CUDA_REV_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct tpgp_cuda_context tpgp_cuda_context;
typedef enum {
    TPGP_CUDA_OK = 0,
    TPGP_CUDA_EINVAL,
    TPGP_CUDA_ENOMEM,
    TPGP_CUDA_EDEVICE,
    TPGP_CUDA_ENUMERIC
} tpgp_cuda_status;

/* 1: this library carries the sm_103a kernels.  It reports build capability,
 * not device availability.  Device indices follow CUDA_VISIBLE_DEVICES; there
 * is no CPU fallback. */
int tpgp_cuda_compiled(void);

/* Creates a context (stream, mutex, persistent scratch) on one device.
 * Returns NULL with a message for a missing or invalid device. */
tpgp_cuda_context *tpgp_cuda_create(int device_index, char *error, size_t error_capacity);

/* Releases the context.  Must not overlap a call that uses it. */
void tpgp_cuda_destroy(tpgp_cuda_context *context);

/* "<device name> (sm_XY)", or "unavailable" for NULL. */
const char *tpgp_cuda_device_name(const tpgp_cuda_context *context);

/* Raw two-child branch of `count` terms (host arrays, caller-owned,
 * disjoint).  Slots 2k and 2k+1 follow the serial engine's order: commuting
 * P gives (P, v, 0) and (P, 0, 0); anticommuting P gives (P, RN(v c), rc')
 * and (P xor Q, sign * RN(v s), rs').  c, s, rc, rs come from the host; no
 * trigonometry runs on the GPU.  With enclose = 1 the radii follow the
 * serial engine's upward-rounded formulas, otherwise they are zero.
 * Statuses: EINVAL for invalid dimensions, sites, generator, factors,
 * overlapping or NULL arrays, size overflow or nonzero padding bits;
 * ENUMERIC for nonfinite inputs or outputs; ENOMEM for device allocation
 * failure; EDEVICE for any other CUDA failure.  Empty input accepts NULL
 * arrays.  Outputs are valid only on success.  Calls sharing a context are
 * serialised; device scratch persists and grows. */
tpgp_cuda_status tpgp_cuda_branches(tpgp_cuda_context *context, const uint64_t *keys,
                                    const double *values, size_t count, size_t n_words,
                                    size_t n_spins, size_t i, size_t j, unsigned qi, unsigned qj,
                                    double c, double s, double rc, double rs, int enclose,
                                    uint64_t *output_keys, double *output_values,
                                    double *output_radii, char *error, size_t error_capacity);

/* Allocation-free variant of tpgp_cuda_branches (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc -- code inside a host
 * allocator or a real-time section, plugins whose host application owns all
 * device memory, processes whose device memory another runtime has reserved:
 * the device staging buffers live in a 16 MiB array that the library's
 * module holds on every GPU that loads it, until exit.  No context is
 * needed; device_index (0..63) selects the GPU and the caller's current
 * device is restored.  Arguments, slot order, statuses and outputs are those
 * of tpgp_cuda_branches; a batch whose staging exceeds the array,
 * (24*n_words + 40)*count + 96 bytes > 16 MiB, is rejected with EINVAL and a
 * message (split it).  Every call looks up the array's device address with
 * that device current (after a device reset the module, and the array, may
 * sit elsewhere); the first call on a device, and the first after a reset,
 * loads the module, so make it before any stream capture.  The call runs on
 * the legacy default stream: it waits for, and holds up, other work on that
 * stream and on blocking streams of the process, and it cannot run while a
 * global-mode stream capture is open on any thread.  Every call on a device
 * shares the array and keeps the previous call's contents (the failure flag
 * is cleared per call); calls that overlapped on the GPU would race, so this
 * entry point serializes its callers with a process-wide lock and returns
 * only after its copies completed. */
tpgp_cuda_status tpgp_cuda_branches_static(int device_index, const uint64_t *keys,
                                           const double *values, size_t count, size_t n_words,
                                           size_t n_spins, size_t i, size_t j, unsigned qi,
                                           unsigned qj, double c, double s, double rc, double rs,
                                           int enclose, uint64_t *output_keys,
                                           double *output_values, double *output_radii,
                                           char *error, size_t error_capacity);

#ifdef __cplusplus
}
#endif
#endif
