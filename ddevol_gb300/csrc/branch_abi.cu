// Reference-compatible CUDA branch backend (include/tpgp_cuda_rev.h).
//
// Contract (DDevol engine/include/tpgp_cuda_rev.h:9-48, the statuses and
// argument rules its engine relies on at engine/src/tpgp_rev.c:622-640):
// host arrays in, two raw children per term out in the serial engine's slot
// order, trigonometric factors from the host, persistent device scratch per
// context, calls on one context serialised, the caller's current device
// restored.  The kernel is written for sm_103a: one thread per term, keys of
// one or two words move as single 64/128-bit vector accesses, a term's two
// coefficients and two radii are written as one 16-byte store each, and
// failure flags are reduced per warp (ballot) before one atomic.
//
// Host side: a call is first turned into a BranchPlan (every argument rule
// checked, byte sizes computed without overflow); the plan fixes the
// staging layout on the device; a StepRunner then issues the transfers and
// the launch on one stream and stops at the first CUDA error.  The context
// path stages through a growing DeviceScratch; the allocation-free path
// stages through a static device array.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdarg>
#include <mutex>

#include "../../include/tpgp_cuda_rev.h"
#include "common.cuh"

static_assert(sizeof(double) == 8 && DBL_MANT_DIG == 53 && FLT_RADIX == 2,
              "the branch backend requires IEEE binary64");


namespace {

using tg::rounding_radius;  // the serial engine's round_radius (engine/src/tpgp_rev.c:37-42)

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


// ============================================================ host side
namespace {

// Writes the caller's message buffer (always NUL-terminated, may be NULL).
class Report {
  public:
    Report(char* buffer, size_t capacity) : buf_(buffer), cap_(capacity) {
        if (buf_ && cap_) buf_[0] = '\0';
    }
    tpgp_cuda_status fail(tpgp_cuda_status status, const char* format, ...) {
        if (buf_ && cap_) {
            va_list args;
            va_start(args, format);
            std::vsnprintf(buf_, cap_, format, args);
            va_end(args);
        }
        return status;
    }
    // Allocation failures map to ENOMEM, every other CUDA error to EDEVICE.
    tpgp_cuda_status cuda(cudaError_t code, const char* stage) {
        return fail(code == cudaErrorMemoryAllocation ? TPGP_CUDA_ENOMEM : TPGP_CUDA_EDEVICE,
                    "tpgp_cuda: %s failed (%s)", stage, cudaGetErrorString(code));
    }

  private:
    char* buf_;
    size_t cap_;
};

// A validated call: geometry, generator, factors and byte sizes.
struct BranchPlan {
    size_t count = 0, words = 0, spins = 0, i = 0, j = 0;
    unsigned qi = 0, qj = 0;
    double c = 0, s = 0, rc = 0, rs = 0;
    int enclose = 0;
    size_t key_bytes = 0;    // count * words * 8 (input keys)
    size_t value_bytes = 0;  // count * 8 (input coefficients)
};

bool product(size_t a, size_t b, size_t& out) {
    if (b != 0 && a > SIZE_MAX / b) return false;
    out = a * b;
    return true;
}

bool intersects(const void* a, size_t a_bytes, const void* b, size_t b_bytes) {
    const uintptr_t pa = reinterpret_cast<uintptr_t>(a), pb = reinterpret_cast<uintptr_t>(b);
    if (a_bytes > UINTPTR_MAX - pa || b_bytes > UINTPTR_MAX - pb) return true;  // wraps: reject
    return pa < pb + b_bytes && pb < pa + a_bytes;
}

// The geometry and generator rules (checked before anything else, also for
// an empty call): at least two spins, words = ceil(spins / 32), two distinct
// sites below spins, Pauli labels 0..3, finite factors, non-negative
// enclosure radii, enclose 0 or 1.
bool valid_geometry(size_t words, size_t spins, size_t i, size_t j, unsigned qi, unsigned qj,
                    double c, double s, double rc, double rs, int enclose) {
    const bool sizes = spins >= 2 && words == (spins + 31) / 32;
    const bool sites = i < spins && j < spins && i != j;
    const bool labels = qi <= 3 && qj <= 3;
    const bool factors = std::isfinite(c) && std::isfinite(s) && std::isfinite(rc) &&
                         std::isfinite(rs) && rc >= 0 && rs >= 0;
    return sizes && sites && labels && factors && (enclose == 0 || enclose == 1);
}

// Fills `plan` for a non-empty call after valid_geometry: rejects NULL
// arrays, byte counts that overflow, and overlapping host arrays.
tpgp_cuda_status plan_arrays(BranchPlan& plan, const uint64_t* keys, const double* values,
                             const uint64_t* out_keys, const double* out_values,
                             const double* out_radii, Report& report) {
    // every byte count below (staging is at most 3 key_bytes + 5 value_bytes
    // + 96) stays below SIZE_MAX when key_bytes and value_bytes are below SIZE_MAX / 16
    size_t key_words = 0, child_key_bytes = 0, child_value_bytes = 0, headroom = 0;
    const bool sized = product(plan.count, plan.words, key_words) &&
                       product(key_words, 8, plan.key_bytes) &&
                       product(plan.count, 8, plan.value_bytes) &&
                       product(plan.key_bytes, 16, headroom) &&
                       product(plan.value_bytes, 16, headroom);
    child_key_bytes = 2 * plan.key_bytes;
    child_value_bytes = 2 * plan.value_bytes;
    if (!keys || !values || !out_keys || !out_values || !out_radii)
        return report.fail(TPGP_CUDA_EINVAL, "tpgp_cuda: %zu terms but a NULL array", plan.count);
    if (!sized)
        return report.fail(TPGP_CUDA_EINVAL, "tpgp_cuda: %zu terms of %zu words overflow size_t",
                           plan.count, plan.words);
    const void* arrays[5] = {keys, values, out_keys, out_values, out_radii};
    const size_t bytes[5] = {plan.key_bytes, plan.value_bytes, child_key_bytes,
                             child_value_bytes, child_value_bytes};
    for (int a = 0; a < 5; ++a)
        for (int b = a + 1; b < 5; ++b)
            if (intersects(arrays[a], bytes[a], arrays[b], bytes[b]))
                return report.fail(TPGP_CUDA_EINVAL,
                                   "tpgp_cuda: host arrays %d and %d overlap (inputs keys, "
                                   "values; outputs keys, values, radii)", a, b);
    return TPGP_CUDA_OK;
}

// Device staging of one call, 16-byte aligned regions in one block:
// children's keys, values and radii, the input keys and values, the flag.
struct Staging {
    size_t child_keys, child_values, child_radii, in_keys, in_values, flag, bytes;
    explicit Staging(const BranchPlan& p) {
        auto next = [](size_t at, size_t len) { return (at + len + 15) & ~size_t(15); };
        child_keys = 0;
        child_values = next(child_keys, 2 * p.key_bytes);
        child_radii = next(child_values, 2 * p.value_bytes);
        in_keys = next(child_radii, 2 * p.value_bytes);
        in_values = next(in_keys, p.key_bytes);
        flag = next(in_values, p.value_bytes);
        bytes = flag + 16;
    }
};

// Selects a device for the lifetime of the object and puts the caller's
// current device back (restore() reports a failure to do so).
class DeviceScope {
  public:
    cudaError_t enter(int device) {
        cudaError_t e = cudaGetDevice(&previous_);
        if (e == cudaSuccess) e = cudaSetDevice(device);
        active_ = e == cudaSuccess;
        return e;
    }
    cudaError_t restore() {
        if (!active_) return cudaSuccess;
        active_ = false;
        return cudaSetDevice(previous_);
    }
    ~DeviceScope() { restore(); }

  private:
    int previous_ = 0;
    bool active_ = false;
};

// Growing device allocation kept between calls (nothing lives in it across
// calls, so growing frees the old block before allocating the new one).
class DeviceScratch {
  public:
    cudaError_t reserve(size_t bytes) {
        if (bytes <= bytes_) return cudaSuccess;
        release();
        cudaError_t e = cudaMalloc(&ptr_, bytes);
        if (e != cudaSuccess) {
            ptr_ = nullptr;
            return e;
        }
        bytes_ = bytes;
        return cudaSuccess;
    }
    void release() {
        if (ptr_) cudaFree(ptr_);
        ptr_ = nullptr;
        bytes_ = 0;
    }
    unsigned char* data() const { return static_cast<unsigned char*>(ptr_); }

  private:
    void* ptr_ = nullptr;
    size_t bytes_ = 0;
};

// Runs CUDA calls in order until the first error, which it reports.
class StepRunner {
  public:
    explicit StepRunner(Report& report) : report_(report) {}
    template <class Call>
    StepRunner& then(const char* stage, Call&& call) {
        if (status_ == TPGP_CUDA_OK) {
            const cudaError_t e = call();
            if (e != cudaSuccess) status_ = report_.cuda(e, stage);
        }
        return *this;
    }
    bool ok() const { return status_ == TPGP_CUDA_OK; }
    tpgp_cuda_status status() const { return status_; }

  private:
    Report& report_;
    tpgp_cuda_status status_ = TPGP_CUDA_OK;
};

void launch_branch(const BranchPlan& p, unsigned char* base, const Staging& at, int sms,
                   cudaStream_t stream) {
    const size_t blocks_wanted = (p.count + 255) / 256, blocks_max = (size_t)std::max(sms, 1) * 16;
    const unsigned blocks = (unsigned)std::min(blocks_wanted, blocks_max);
    auto* ck = reinterpret_cast<uint64_t*>(base + at.child_keys);
    auto* cv = reinterpret_cast<double*>(base + at.child_values);
    auto* cr = reinterpret_cast<double*>(base + at.child_radii);
    auto* ik = reinterpret_cast<const uint64_t*>(base + at.in_keys);
    auto* iv = reinterpret_cast<const double*>(base + at.in_values);
    auto* flag = reinterpret_cast<unsigned*>(base + at.flag);
#define TPGP_BRANCH_LAUNCH(W)                                                                    \
    k_branch<W><<<blocks, 256, 0, stream>>>(ik, iv, p.count, p.words, p.spins, p.i, p.j, p.qi,   \
                                            p.qj, p.c, p.s, p.rc, p.rs, p.enclose, ck, cv, cr,   \
                                            flag)
    if (p.words == 1) TPGP_BRANCH_LAUNCH(1);
    else if (p.words == 2) TPGP_BRANCH_LAUNCH(2);
    else TPGP_BRANCH_LAUNCH(0);
#undef TPGP_BRANCH_LAUNCH
}

// Stages one planned call through `base` on `stream`: inputs up, flag
// cleared, kernel, then the flag and all children down in one go and a
// single wait.  The children reach the caller's arrays even when the flag
// reports a failure; the contract makes outputs valid only on success.
tpgp_cuda_status run_branch(const BranchPlan& p, unsigned char* base, int sms, cudaStream_t stream,
                            const uint64_t* keys, const double* values, uint64_t* out_keys,
                            double* out_values, double* out_radii, Report& report) {
    const Staging at(p);
    unsigned flag = 0;
    StepRunner run(report);
    run.then("input key upload", [&] {
           return cudaMemcpyAsync(base + at.in_keys, keys, p.key_bytes, cudaMemcpyHostToDevice,
                                  stream);
       })
        .then("input coefficient upload", [&] {
            return cudaMemcpyAsync(base + at.in_values, values, p.value_bytes,
                                   cudaMemcpyHostToDevice, stream);
        })
        .then("failure flag reset", [&] { return cudaMemsetAsync(base + at.flag, 0, 4, stream); })
        .then("branch kernel launch", [&] {
            launch_branch(p, base, at, sms, stream);
            return cudaGetLastError();
        })
        .then("failure flag download", [&] {
            return cudaMemcpyAsync(&flag, base + at.flag, 4, cudaMemcpyDeviceToHost, stream);
        })
        .then("child key download", [&] {
            return cudaMemcpyAsync(out_keys, base + at.child_keys, 2 * p.key_bytes,
                                   cudaMemcpyDeviceToHost, stream);
        })
        .then("child coefficient download", [&] {
            return cudaMemcpyAsync(out_values, base + at.child_values, 2 * p.value_bytes,
                                   cudaMemcpyDeviceToHost, stream);
        })
        .then("child radius download", [&] {
            return cudaMemcpyAsync(out_radii, base + at.child_radii, 2 * p.value_bytes,
                                   cudaMemcpyDeviceToHost, stream);
        })
        .then("branch execution", [&] { return cudaStreamSynchronize(stream); });
    if (!run.ok()) {
        cudaStreamSynchronize(stream);  // nothing may still target the caller's arrays
        return run.status();
    }
    if (flag & 1u)
        return report.fail(TPGP_CUDA_EINVAL,
                           "tpgp_cuda: an input key sets bits above site %zu", p.spins - 1);
    if (flag & 2u)
        return report.fail(TPGP_CUDA_ENUMERIC,
                           "tpgp_cuda: a coefficient, child or radius is not finite");
    return TPGP_CUDA_OK;
}

}  // namespace

struct tpgp_cuda_context {
    int device = 0;
    int sms = 1;
    cudaStream_t stream = nullptr;
    DeviceScratch scratch;
    std::mutex lock;  // serialises calls on this context
    char name[256] = {};
};

extern "C" int tpgp_cuda_compiled(void) { return 1; }

extern "C" tpgp_cuda_context* tpgp_cuda_create(int index, char* error, size_t cap) {
    Report report(error, cap);
    int devices = 0;
    cudaError_t e = cudaGetDeviceCount(&devices);
    if (e != cudaSuccess) {
        report.cuda(e, "device count");
        return nullptr;
    }
    if (index < 0 || index >= devices) {
        report.fail(TPGP_CUDA_EINVAL, "tpgp_cuda: device %d requested, %d visible", index, devices);
        return nullptr;
    }
    cudaDeviceProp prop;
    if ((e = cudaGetDeviceProperties(&prop, index)) != cudaSuccess) {
        report.cuda(e, "device properties");
        return nullptr;
    }
    auto* ctx = new (std::nothrow) tpgp_cuda_context();
    if (!ctx) {
        report.fail(TPGP_CUDA_ENOMEM, "tpgp_cuda: out of host memory for the context");
        return nullptr;
    }
    ctx->device = index;
    ctx->sms = std::max(prop.multiProcessorCount, 1);
    std::snprintf(ctx->name, sizeof(ctx->name), "%.200s (sm_%d%d)", prop.name, prop.major,
                  prop.minor);
    DeviceScope scope;
    if ((e = scope.enter(index)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        report.cuda(e, "stream set-up");
        delete ctx;
        return nullptr;
    }
    if ((e = scope.restore()) != cudaSuccess) {
        report.cuda(e, "restoring the caller's device");
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return nullptr;
    }
    return ctx;
}

extern "C" void tpgp_cuda_destroy(tpgp_cuda_context* ctx) {
    if (!ctx) return;
    {
        DeviceScope scope;
        if (scope.enter(ctx->device) == cudaSuccess) {
            cudaStreamSynchronize(ctx->stream);
            ctx->scratch.release();
            cudaStreamDestroy(ctx->stream);
        }
    }
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
    Report report(error, cap);
    if (!ctx)
        return report.fail(TPGP_CUDA_EINVAL, "tpgp_cuda: NULL context");
    if (!valid_geometry(words, spins, i, j, qi, qj, c, s, rc, rs, enclose))
        return report.fail(TPGP_CUDA_EINVAL,
                           "tpgp_cuda: invalid rotation (spins %zu, words %zu, sites %zu/%zu, "
                           "labels %u/%u, factors or enclose flag)", spins, words, i, j, qi, qj);
    if (count == 0) return TPGP_CUDA_OK;  // NULL arrays are fine for an empty call
    BranchPlan plan;
    plan.count = count, plan.words = words, plan.spins = spins, plan.i = i, plan.j = j;
    plan.qi = qi, plan.qj = qj, plan.c = c, plan.s = s, plan.rc = rc, plan.rs = rs;
    plan.enclose = enclose;
    tpgp_cuda_status st = plan_arrays(plan, keys, values, out_keys, out_values, out_radii, report);
    if (st != TPGP_CUDA_OK) return st;
    std::lock_guard<std::mutex> guard(ctx->lock);
    DeviceScope scope;
    cudaError_t e = scope.enter(ctx->device);
    if (e != cudaSuccess) return report.cuda(e, "device selection");
    if ((e = ctx->scratch.reserve(Staging(plan).bytes)) != cudaSuccess)
        return report.cuda(e, "staging allocation");
    st = run_branch(plan, ctx->scratch.data(), ctx->sms, ctx->stream, keys, values, out_keys,
                    out_values, out_radii, report);
    e = scope.restore();
    if (st == TPGP_CUDA_OK && e != cudaSuccess) return report.cuda(e, "restoring the caller's device");
    return st;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of tpgp_cuda_branches.
//
// Some callers cannot call cudaMalloc: code running inside a host allocator
// or a signal-safe/real-time section, plugins whose host application owns
// all device memory, or processes whose device memory is fully reserved by
// another runtime.  For them the device staging of the branch kernel lives
// in one file-scope array that the library's module brings with it; the
// call itself allocates nothing.  The array's host-side name is not a device
// address, so every call asks the runtime for the address on the selected
// device (cheap once the module is loaded, and never stale after a device
// reset reloaded the module elsewhere).
namespace {

constexpr size_t kStaticScratchBytes = size_t(16) << 20;  // 16 MiB per device
static __device__ __align__(256) unsigned char g_branch_scratch[kStaticScratchBytes];

constexpr int kMaxStaticDevices = 64;
std::mutex g_static_lock;  // every call shares the array: calls are serialised

}  // namespace

extern "C" tpgp_cuda_status tpgp_cuda_branches_static(
    int device_index, const uint64_t* keys, const double* values, size_t count, size_t words,
    size_t spins, size_t i, size_t j, unsigned qi, unsigned qj, double c, double s, double rc,
    double rs, int enclose, uint64_t* out_keys, double* out_values, double* out_radii,
    char* error, size_t cap) {
    Report report(error, cap);
    if (device_index < 0 || device_index >= kMaxStaticDevices)
        return report.fail(TPGP_CUDA_EINVAL, "tpgp_cuda: device index %d outside 0..%d",
                           device_index, kMaxStaticDevices - 1);
    if (!valid_geometry(words, spins, i, j, qi, qj, c, s, rc, rs, enclose))
        return report.fail(TPGP_CUDA_EINVAL,
                           "tpgp_cuda: invalid rotation (spins %zu, words %zu, sites %zu/%zu, "
                           "labels %u/%u, factors or enclose flag)", spins, words, i, j, qi, qj);
    if (count == 0) return TPGP_CUDA_OK;
    BranchPlan plan;
    plan.count = count, plan.words = words, plan.spins = spins, plan.i = i, plan.j = j;
    plan.qi = qi, plan.qj = qj, plan.c = c, plan.s = s, plan.rc = rc, plan.rs = rs;
    plan.enclose = enclose;
    tpgp_cuda_status st = plan_arrays(plan, keys, values, out_keys, out_values, out_radii, report);
    if (st != TPGP_CUDA_OK) return st;
    const size_t need = Staging(plan).bytes;
    if (need > kStaticScratchBytes)
        return report.fail(TPGP_CUDA_EINVAL,
                           "tpgp_cuda: %zu terms need %zu bytes of staging; the allocation-free "
                           "entry point holds at most %zu bytes ((24*n_words + 40) bytes per "
                           "term); split the batch", count, need, kStaticScratchBytes);
    std::lock_guard<std::mutex> guard(g_static_lock);
    int devices = 0;
    cudaError_t e = cudaGetDeviceCount(&devices);
    if (e != cudaSuccess) return report.cuda(e, "device count");
    if (device_index >= devices)
        return report.fail(TPGP_CUDA_EINVAL, "tpgp_cuda: device %d requested, %d visible",
                           device_index, devices);
    DeviceScope scope;
    if ((e = scope.enter(device_index)) != cudaSuccess) return report.cuda(e, "device selection");
    void* base = nullptr;  // the array's address on this device
    if ((e = cudaGetSymbolAddress(&base, g_branch_scratch)) != cudaSuccess)
        return report.cuda(e, "static staging address lookup");
    int sms = 1;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_index)) !=
        cudaSuccess)
        return report.cuda(e, "multiprocessor count");
    // the legacy default stream: no stream to create; the array keeps the
    // previous call's contents, and run_branch clears the failure flag
    st = run_branch(plan, static_cast<unsigned char*>(base), sms, cudaStreamLegacy, keys, values,
                    out_keys, out_values, out_radii, report);
    e = scope.restore();
    if (st == TPGP_CUDA_OK && e != cudaSuccess) return report.cuda(e, "restoring the caller's device");
    return st;
}
