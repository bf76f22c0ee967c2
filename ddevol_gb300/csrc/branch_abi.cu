// Reference-compatible CUDA branch backend (include/tpgp_cuda_rev.h).
//
// Same contract as DDevol engine/src/cuda_rev.cu:117-272: host arrays in,
// two raw children per term out in the serial engine's slot order, host
// trigonometric factors, persistent device scratch, calls on one context
// serialised.  The kernel is written for sm_103a: one thread per term, keys
// of one or two words move as single 64/128-bit vector accesses, a term's
// two coefficients and two radii are written as one 16-byte store each, and
// failure flags are reduced per warp (ballot) before one atomic.
#include <cuda_runtime.h>

#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "../../include/tpgp_cuda_rev.h"
#include "common.cuh"

static_assert(sizeof(double) == 8 && DBL_MANT_DIG == 53 && FLT_RADIX == 2,
              "the branch backend requires IEEE binary64");

struct tpgp_cuda_context {
    int device;
    int sms;
    cudaStream_t stream;
    void* scratch;
    size_t scratch_bytes;
    std::mutex lock;
    char name[256];
};

namespace {

void set_message(char* error, size_t cap, const char* text) {
    if (error && cap) std::snprintf(error, cap, "%s", text);
}
tpgp_cuda_status cuda_failure(cudaError_t code, const char* what, char* error, size_t cap) {
    if (error && cap) std::snprintf(error, cap, "%s: %s", what, cudaGetErrorString(code));
    return code == cudaErrorMemoryAllocation ? TPGP_CUDA_ENOMEM : TPGP_CUDA_EDEVICE;
}
bool mul_ok(size_t a, size_t b, size_t* out) {
    if (b && a > SIZE_MAX / b) return false;
    *out = a * b;
    return true;
}
bool add_ok(size_t a, size_t b, size_t* out) {
    if (a > SIZE_MAX - b) return false;
    *out = a + b;
    return true;
}
bool ranges_overlap(const void* a, size_t as, const void* b, size_t bs) {
    const uintptr_t x = (uintptr_t)a, y = (uintptr_t)b;
    if (as > UINTPTR_MAX - x || bs > UINTPTR_MAX - y) return true;
    return x < y + bs && y < x + as;
}

// Largest |x - neighbour| over the two adjacent binary64 values: the
// rounding radius of the serial engine (engine/src/tpgp_rev.c:37-42).
__device__ __forceinline__ double rounding_radius(double x) {
    if (!tg::is_finite(x)) return __longlong_as_double(0x7ff0000000000000ll);
    const double up = tg::next_up(x), down = tg::negate(tg::next_up(tg::negate(x)));
    const double a = fabs(__dsub_rn(up, x)), b = fabs(__dsub_rn(x, down));
    return a > b ? a : b;
}

// W > 0: keys of exactly W words held in registers; W == 0: any word count.
template <int W>
__global__ void __launch_bounds__(256)
    k_branch(const uint64_t* __restrict__ keys, const double* __restrict__ values, size_t count,
             size_t words, size_t spins, size_t i, size_t j, unsigned qi, unsigned qj, double c,
             double s, double rc, double rs, int enclose, uint64_t* __restrict__ out_keys,
             double* __restrict__ out_values, double* __restrict__ out_radii,
             unsigned* __restrict__ failure) {
    const size_t nw = W > 0 ? (size_t)W : words;
    const size_t rem = spins % 32;
    const int iw = (int)(i / 32), is = (int)(2 * (i % 32));
    const int jw = (int)(j / 32), js = (int)(2 * (j % 32));
    const uint64_t mi = (uint64_t)qi << is, mj = (uint64_t)qj << js;
    const size_t stride = (size_t)blockDim.x * gridDim.x;
    for (size_t base = (size_t)blockIdx.x * blockDim.x; base < count; base += stride) {
        const size_t k = base + threadIdx.x;
        unsigned flags = 0;
        if (k < count) {
            uint64_t top, wi, wj;
            if constexpr (W == 1) {
                const uint64_t key = __ldg(keys + k);
                top = wi = wj = key;
                reinterpret_cast<ulonglong2*>(out_keys)[k] = make_ulonglong2(key, key);
            } else if constexpr (W == 2) {
                const ulonglong2 key = __ldg(reinterpret_cast<const ulonglong2*>(keys) + k);
                top = key.y;
                wi = iw ? key.y : key.x;
                wj = jw ? key.y : key.x;
                reinterpret_cast<ulonglong2*>(out_keys)[2 * k] = key;
                reinterpret_cast<ulonglong2*>(out_keys)[2 * k + 1] = key;
            } else {
                const uint64_t* kp = keys + k * nw;
                uint64_t* a = out_keys + 2 * k * nw;
                for (size_t w = 0; w < nw; ++w) a[w] = a[nw + w] = kp[w];
                top = kp[nw - 1];
                wi = kp[iw];
                wj = kp[jw];
            }
            if (rem && (top >> (2 * rem))) flags |= 1u;
            const unsigned pi = tg::site_symbol(wi, is), pj = tg::site_symbol(wj, js);
            const bool anti = tg::anticommutes(qi, pi) != tg::anticommutes(qj, pj);
            const double v = __ldg(values + k);
            if (!tg::is_finite(v)) flags |= 2u;
            if (!anti) {
                reinterpret_cast<double2*>(out_values)[k] = make_double2(v, 0.0);
                reinterpret_cast<double2*>(out_radii)[k] = make_double2(0.0, 0.0);
            } else {
                const bool plus = ((tg::phase_exponent(qi, pi) + tg::phase_exponent(qj, pj)) & 3u) == 1u;
                // flip the two sites of the second child
                if constexpr (W == 1) {
                    out_keys[2 * k + 1] = wi ^ mi ^ mj;
                } else {
                    uint64_t* d = out_keys + (2 * k + 1) * nw;
                    d[iw] ^= mi;
                    d[jw] ^= mj;
                }
                const double x = __dmul_rn(v, c), y = __dmul_rn(v, s);
                double r0 = 0.0, r1 = 0.0;
                if (enclose) {
                    r0 = tg::up_add(tg::up_mul(tg::abs_of(v), rc), rounding_radius(x));
                    r1 = tg::up_add(tg::up_mul(tg::abs_of(v), rs), rounding_radius(y));
                }
                reinterpret_cast<double2*>(out_values)[k] = make_double2(x, plus ? y : tg::negate(y));
                reinterpret_cast<double2*>(out_radii)[k] = make_double2(r0, r1);
                if (!tg::is_finite(x) || !tg::is_finite(y) || !tg::is_finite(r0) || !tg::is_finite(r1))
                    flags |= 2u;
            }
        }
        const unsigned any1 = __ballot_sync(0xffffffffu, flags & 1u);
        const unsigned any2 = __ballot_sync(0xffffffffu, flags & 2u);
        if ((threadIdx.x & 31) == 0 && (any1 | any2))
            atomicOr(failure, (any1 ? 1u : 0u) | (any2 ? 2u : 0u));
    }
}

}  // namespace

extern "C" int tpgp_cuda_compiled(void) { return 1; }

extern "C" tpgp_cuda_context* tpgp_cuda_create(int index, char* error, size_t cap) {
    set_message(error, cap, "");
    int count = 0, previous = 0;
    cudaError_t code = cudaGetDeviceCount(&count);
    if (code != cudaSuccess) {
        cuda_failure(code, "CUDA device discovery", error, cap);
        return nullptr;
    }
    if (index < 0 || index >= count) {
        set_message(error, cap, "Requested CUDA device index is unavailable.");
        return nullptr;
    }
    if ((code = cudaGetDevice(&previous)) != cudaSuccess) {
        cuda_failure(code, "CUDA current-device query", error, cap);
        return nullptr;
    }
    if ((code = cudaSetDevice(index)) != cudaSuccess) {
        cuda_failure(code, "CUDA device selection", error, cap);
        return nullptr;
    }
    cudaDeviceProp prop;
    if ((code = cudaGetDeviceProperties(&prop, index)) != cudaSuccess) {
        cuda_failure(code, "CUDA device properties", error, cap);
        cudaSetDevice(previous);
        return nullptr;
    }
    auto* ctx = new (std::nothrow) tpgp_cuda_context();
    if (!ctx) {
        set_message(error, cap, "Could not allocate the CUDA host context.");
        cudaSetDevice(previous);
        return nullptr;
    }
    ctx->device = index;
    ctx->sms = prop.multiProcessorCount > 0 ? prop.multiProcessorCount : 1;
    std::snprintf(ctx->name, sizeof(ctx->name), "%s (sm_%d%d)", prop.name, prop.major, prop.minor);
    if ((code = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        cuda_failure(code, "CUDA stream creation", error, cap);
        delete ctx;
        cudaSetDevice(previous);
        return nullptr;
    }
    if ((code = cudaSetDevice(previous)) != cudaSuccess) {
        cuda_failure(code, "CUDA previous-device restoration", error, cap);
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return nullptr;
    }
    return ctx;
}

extern "C" void tpgp_cuda_destroy(tpgp_cuda_context* ctx) {
    if (!ctx) return;
    int previous = ctx->device;
    cudaGetDevice(&previous);
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->scratch) cudaFree(ctx->scratch);
    cudaStreamDestroy(ctx->stream);
    cudaSetDevice(previous);
    delete ctx;
}

extern "C" const char* tpgp_cuda_device_name(const tpgp_cuda_context* ctx) {
    return ctx ? ctx->name : "unavailable";
}

extern "C" tpgp_cuda_status tpgp_cuda_branches(tpgp_cuda_context* ctx, const uint64_t* keys,
                                               const double* values, size_t count, size_t words,
                                               size_t spins, size_t i, size_t j, unsigned qi,
                                               unsigned qj, double c, double s, double rc,
                                               double rs, int enclose, uint64_t* out_keys,
                                               double* out_values, double* out_radii,
                                               char* error, size_t cap) {
    set_message(error, cap, "");
    // argument checks of engine/src/cuda_rev.cu:180-203, in the same order
    if (!ctx || spins < 2 || words != spins / 32 + (spins % 32 != 0) || i >= spins ||
        j >= spins || i == j || qi > 3 || qj > 3 || !std::isfinite(c) || !std::isfinite(s) ||
        !std::isfinite(rc) || !std::isfinite(rs) || rc < 0 || rs < 0 ||
        (enclose != 0 && enclose != 1)) {
        set_message(error, cap,
                    "Invalid CUDA branch dimensions, sites, generator, or trigonometric enclosure.");
        return TPGP_CUDA_EINVAL;
    }
    if (!count) return TPGP_CUDA_OK;
    size_t key_bytes, value_bytes, out_key_bytes, out_value_bytes, total, t;
    if (!keys || !values || !out_keys || !out_values || !out_radii || !mul_ok(count, words, &t) ||
        !mul_ok(t, sizeof(uint64_t), &key_bytes) || !mul_ok(count, sizeof(double), &value_bytes) ||
        !mul_ok(key_bytes, 2, &out_key_bytes) || !mul_ok(value_bytes, 2, &out_value_bytes) ||
        !mul_ok(key_bytes, 3, &total) || !mul_ok(value_bytes, 5, &t) || !add_ok(total, t, &total) ||
        !add_ok(total, 64, &total)) {
        set_message(error, cap, "Null CUDA array or packed-branch allocation size overflow.");
        return TPGP_CUDA_EINVAL;
    }
    const void* arrays[] = {keys, values, out_keys, out_values, out_radii};
    const size_t lengths[] = {key_bytes, value_bytes, out_key_bytes, out_value_bytes,
                              out_value_bytes};
    for (int x = 0; x < 5; ++x)
        for (int y = x + 1; y < 5; ++y)
            if (ranges_overlap(arrays[x], lengths[x], arrays[y], lengths[y])) {
                set_message(error, cap, "CUDA input/output arrays must be disjoint.");
                return TPGP_CUDA_EINVAL;
            }
    std::lock_guard<std::mutex> guard(ctx->lock);
    tpgp_cuda_status result = TPGP_CUDA_OK;
    int previous = ctx->device;
    cudaError_t code = cudaGetDevice(&previous);
    if (code != cudaSuccess) result = cuda_failure(code, "CUDA current-device query", error, cap);
    if (result == TPGP_CUDA_OK && (code = cudaSetDevice(ctx->device)) != cudaSuccess)
        result = cuda_failure(code, "CUDA device selection", error, cap);
    if (result == TPGP_CUDA_OK && total > ctx->scratch_bytes) {
        // nothing lives in the scratch between calls: release before growing
        if (ctx->scratch) {
            code = cudaFree(ctx->scratch);
            ctx->scratch = nullptr;
            ctx->scratch_bytes = 0;
            if (code != cudaSuccess) result = cuda_failure(code, "CUDA scratch release", error, cap);
        }
        if (result == TPGP_CUDA_OK) {
            if ((code = cudaMalloc(&ctx->scratch, total)) != cudaSuccess) {
                ctx->scratch = nullptr;
                result = cuda_failure(code, "CUDA persistent scratch allocation", error, cap);
            } else {
                ctx->scratch_bytes = total;
            }
        }
    }
    if (result == TPGP_CUDA_OK) {
        // 16-byte aligned sub-buffers: out keys, out values, out radii, in keys, in values, flags
        unsigned char* base = static_cast<unsigned char*>(ctx->scratch);
        auto align16 = [](size_t x) { return (x + 15) & ~size_t(15); };
        size_t off = 0;
        uint64_t* d_out_keys = reinterpret_cast<uint64_t*>(base + off);
        off = align16(off + out_key_bytes);
        double* d_out_values = reinterpret_cast<double*>(base + off);
        off = align16(off + out_value_bytes);
        double* d_out_radii = reinterpret_cast<double*>(base + off);
        off = align16(off + out_value_bytes);
        uint64_t* d_keys = reinterpret_cast<uint64_t*>(base + off);
        off = align16(off + key_bytes);
        double* d_values = reinterpret_cast<double*>(base + off);
        off = align16(off + value_bytes);
        unsigned* d_failure = reinterpret_cast<unsigned*>(base + off);
        unsigned failure = 0;
#define STEP(call, what)                                                      \
    do {                                                                      \
        if (result == TPGP_CUDA_OK) {                                         \
            code = (call);                                                    \
            if (code != cudaSuccess) result = cuda_failure(code, what, error, cap); \
        }                                                                     \
    } while (0)
        STEP(cudaMemcpyAsync(d_keys, keys, key_bytes, cudaMemcpyHostToDevice, ctx->stream),
             "CUDA input-key transfer");
        STEP(cudaMemcpyAsync(d_values, values, value_bytes, cudaMemcpyHostToDevice, ctx->stream),
             "CUDA input-coefficient transfer");
        STEP(cudaMemsetAsync(d_failure, 0, sizeof(unsigned), ctx->stream), "CUDA status reset");
        if (result == TPGP_CUDA_OK) {
            const size_t want = (count + 255) / 256;
            const size_t cap_blocks = (size_t)ctx->sms * 16;
            const unsigned blocks = (unsigned)(want < cap_blocks ? want : cap_blocks);
            if (words == 1)
                k_branch<1><<<blocks, 256, 0, ctx->stream>>>(
                    d_keys, d_values, count, words, spins, i, j, qi, qj, c, s, rc, rs, enclose,
                    d_out_keys, d_out_values, d_out_radii, d_failure);
            else if (words == 2)
                k_branch<2><<<blocks, 256, 0, ctx->stream>>>(
                    d_keys, d_values, count, words, spins, i, j, qi, qj, c, s, rc, rs, enclose,
                    d_out_keys, d_out_values, d_out_radii, d_failure);
            else
                k_branch<0><<<blocks, 256, 0, ctx->stream>>>(
                    d_keys, d_values, count, words, spins, i, j, qi, qj, c, s, rc, rs, enclose,
                    d_out_keys, d_out_values, d_out_radii, d_failure);
            STEP(cudaGetLastError(), "CUDA branch-kernel launch");
        }
        STEP(cudaMemcpyAsync(&failure, d_failure, sizeof(unsigned), cudaMemcpyDeviceToHost,
                             ctx->stream),
             "CUDA status transfer");
        STEP(cudaStreamSynchronize(ctx->stream), "CUDA branch-kernel execution");
        if (result == TPGP_CUDA_OK && failure) {
            result = (failure & 1u) ? TPGP_CUDA_EINVAL : TPGP_CUDA_ENUMERIC;
            set_message(error, cap,
                        (failure & 1u) ? "CUDA input keys contain nonzero padding bits."
                                       : "CUDA branch arithmetic or coefficients are nonfinite.");
        }
        STEP(cudaMemcpyAsync(out_keys, d_out_keys, out_key_bytes, cudaMemcpyDeviceToHost,
                             ctx->stream),
             "CUDA output-key transfer");
        STEP(cudaMemcpyAsync(out_values, d_out_values, out_value_bytes, cudaMemcpyDeviceToHost,
                             ctx->stream),
             "CUDA output-coefficient transfer");
        STEP(cudaMemcpyAsync(out_radii, d_out_radii, out_value_bytes, cudaMemcpyDeviceToHost,
                             ctx->stream),
             "CUDA output-radius transfer");
        STEP(cudaStreamSynchronize(ctx->stream), "CUDA output completion");
        // drain queued work before the caller may release its arrays
        if (result != TPGP_CUDA_OK) cudaStreamSynchronize(ctx->stream);
#undef STEP
    }
    code = cudaSetDevice(previous);
    if (result == TPGP_CUDA_OK && code != cudaSuccess)
        result = cuda_failure(code, "CUDA previous-device restoration", error, cap);
    return result;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of tpgp_cuda_branches.
//
// Some callers cannot call cudaMalloc: code running inside a host allocator
// or a signal-safe/real-time section, plugins whose host application owns
// all device memory, or processes whose device memory is fully reserved by
// another runtime.  For them the device staging buffers of the branch kernel
// (input keys/values, output keys/values/radii, failure flag) live in one
// file-scope array that the library's module brings with it; the call itself
// allocates nothing.
namespace {

constexpr size_t kStaticScratchBytes = size_t(16) << 20;  // 16 MiB per device
static __device__ __align__(256) unsigned char g_branch_scratch[kStaticScratchBytes];

constexpr int kMaxStaticDevices = 64;
std::mutex g_static_lock;                                 // serializes every call
void* g_static_address[kMaxStaticDevices] = {nullptr};    // device address, per device

}  // namespace

extern "C" tpgp_cuda_status tpgp_cuda_branches_static(
    int device_index, const uint64_t* keys, const double* values, size_t count, size_t words,
    size_t spins, size_t i, size_t j, unsigned qi, unsigned qj, double c, double s, double rc,
    double rs, int enclose, uint64_t* out_keys, double* out_values, double* out_radii,
    char* error, size_t cap) {
    set_message(error, cap, "");
    // the same argument checks, in the same order, as tpgp_cuda_branches
    if (device_index < 0 || device_index >= kMaxStaticDevices || spins < 2 ||
        words != spins / 32 + (spins % 32 != 0) || i >= spins || j >= spins || i == j ||
        qi > 3 || qj > 3 || !std::isfinite(c) || !std::isfinite(s) || !std::isfinite(rc) ||
        !std::isfinite(rs) || rc < 0 || rs < 0 || (enclose != 0 && enclose != 1)) {
        set_message(error, cap,
                    "Invalid CUDA branch device, dimensions, sites, generator, or trigonometric enclosure.");
        return TPGP_CUDA_EINVAL;
    }
    if (!count) return TPGP_CUDA_OK;
    size_t key_bytes, value_bytes, out_key_bytes, out_value_bytes, total, t;
    if (!keys || !values || !out_keys || !out_values || !out_radii || !mul_ok(count, words, &t) ||
        !mul_ok(t, sizeof(uint64_t), &key_bytes) || !mul_ok(count, sizeof(double), &value_bytes) ||
        !mul_ok(key_bytes, 2, &out_key_bytes) || !mul_ok(value_bytes, 2, &out_value_bytes) ||
        !mul_ok(key_bytes, 3, &total) || !mul_ok(value_bytes, 5, &t) || !add_ok(total, t, &total) ||
        !add_ok(total, 128, &total)) {
        set_message(error, cap, "Null CUDA array or packed-branch size overflow.");
        return TPGP_CUDA_EINVAL;
    }
    if (total > kStaticScratchBytes) {
        if (error && cap)
            std::snprintf(error, cap,
                          "Batch needs %zu bytes of staging; the allocation-free entry point holds "
                          "at most %zu bytes ((24*n_words + 40) bytes per term). Split the batch.",
                          total, kStaticScratchBytes);
        return TPGP_CUDA_EINVAL;
    }
    const void* arrays[] = {keys, values, out_keys, out_values, out_radii};
    const size_t lengths[] = {key_bytes, value_bytes, out_key_bytes, out_value_bytes,
                              out_value_bytes};
    for (int x = 0; x < 5; ++x)
        for (int y = x + 1; y < 5; ++y)
            if (ranges_overlap(arrays[x], lengths[x], arrays[y], lengths[y])) {
                set_message(error, cap, "CUDA input/output arrays must be disjoint.");
                return TPGP_CUDA_EINVAL;
            }
    std::lock_guard<std::mutex> guard(g_static_lock);
    tpgp_cuda_status result = TPGP_CUDA_OK;
    int previous = 0, count_dev = 0;
    cudaError_t code = cudaGetDeviceCount(&count_dev);
    if (code != cudaSuccess) return cuda_failure(code, "CUDA device discovery", error, cap);
    if (device_index >= count_dev) {
        set_message(error, cap, "Requested CUDA device index is unavailable.");
        return TPGP_CUDA_EINVAL;
    }
    if ((code = cudaGetDevice(&previous)) != cudaSuccess)
        return cuda_failure(code, "CUDA current-device query", error, cap);
    if ((code = cudaSetDevice(device_index)) != cudaSuccess)
        return cuda_failure(code, "CUDA device selection", error, cap);
    // set-up, once per device, with that device current: the host-side name
    // of the array is not a device address, so ask the runtime for it
    if (!g_static_address[device_index]) {
        void* ptr = nullptr;
        code = cudaGetSymbolAddress(&ptr, g_branch_scratch);
        if (code != cudaSuccess) {
            result = cuda_failure(code, "CUDA static scratch address", error, cap);
            cudaSetDevice(previous);
            return result;
        }
        g_static_address[device_index] = ptr;
    }
    unsigned char* base = static_cast<unsigned char*>(g_static_address[device_index]);
    auto align16 = [](size_t x) { return (x + 15) & ~size_t(15); };
    size_t off = 0;
    uint64_t* d_out_keys = reinterpret_cast<uint64_t*>(base + off);
    off = align16(off + out_key_bytes);
    double* d_out_values = reinterpret_cast<double*>(base + off);
    off = align16(off + out_value_bytes);
    double* d_out_radii = reinterpret_cast<double*>(base + off);
    off = align16(off + out_value_bytes);
    uint64_t* d_keys = reinterpret_cast<uint64_t*>(base + off);
    off = align16(off + key_bytes);
    double* d_values = reinterpret_cast<double*>(base + off);
    off = align16(off + value_bytes);
    unsigned* d_failure = reinterpret_cast<unsigned*>(base + off);
    unsigned failure = 0;
#define STEP(call, what)                                                      \
    do {                                                                      \
        if (result == TPGP_CUDA_OK) {                                         \
            code = (call);                                                    \
            if (code != cudaSuccess) result = cuda_failure(code, what, error, cap); \
        }                                                                     \
    } while (0)
    STEP(cudaMemcpy(d_keys, keys, key_bytes, cudaMemcpyHostToDevice), "CUDA input-key transfer");
    STEP(cudaMemcpy(d_values, values, value_bytes, cudaMemcpyHostToDevice),
         "CUDA input-coefficient transfer");
    // the array keeps the previous call's contents: the failure flag must start at zero
    STEP(cudaMemset(d_failure, 0, sizeof(unsigned)), "CUDA status reset");
    if (result == TPGP_CUDA_OK) {
        int sms = 1;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_index);
        const size_t want = (count + 255) / 256, cap_blocks = (size_t)(sms > 0 ? sms : 1) * 16;
        const unsigned blocks = (unsigned)(want < cap_blocks ? want : cap_blocks);
        if (words == 1)
            k_branch<1><<<blocks, 256>>>(d_keys, d_values, count, words, spins, i, j, qi, qj, c,
                                         s, rc, rs, enclose, d_out_keys, d_out_values,
                                         d_out_radii, d_failure);
        else if (words == 2)
            k_branch<2><<<blocks, 256>>>(d_keys, d_values, count, words, spins, i, j, qi, qj, c,
                                         s, rc, rs, enclose, d_out_keys, d_out_values,
                                         d_out_radii, d_failure);
        else
            k_branch<0><<<blocks, 256>>>(d_keys, d_values, count, words, spins, i, j, qi, qj, c,
                                         s, rc, rs, enclose, d_out_keys, d_out_values,
                                         d_out_radii, d_failure);
        STEP(cudaGetLastError(), "CUDA branch-kernel launch");
    }
    STEP(cudaMemcpy(&failure, d_failure, sizeof(unsigned), cudaMemcpyDeviceToHost),
         "CUDA branch-kernel execution");
    if (result == TPGP_CUDA_OK && failure) {
        result = (failure & 1u) ? TPGP_CUDA_EINVAL : TPGP_CUDA_ENUMERIC;
        set_message(error, cap,
                    (failure & 1u) ? "CUDA input keys contain nonzero padding bits."
                                   : "CUDA branch arithmetic or coefficients are nonfinite.");
    }
    STEP(cudaMemcpy(out_keys, d_out_keys, out_key_bytes, cudaMemcpyDeviceToHost),
         "CUDA output-key transfer");
    STEP(cudaMemcpy(out_values, d_out_values, out_value_bytes, cudaMemcpyDeviceToHost),
         "CUDA output-coefficient transfer");
    STEP(cudaMemcpy(out_radii, d_out_radii, out_value_bytes, cudaMemcpyDeviceToHost),
         "CUDA output-radius transfer");
#undef STEP
    code = cudaSetDevice(previous);
    if (result == TPGP_CUDA_OK && code != cudaSuccess)
        result = cuda_failure(code, "CUDA previous-device restoration", error, cap);
    return result;
}
