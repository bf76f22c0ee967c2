// Shared device code for the GB300 Pauli-propagation kernels.
//
// Keys follow the reference map layout (DDevol engine/include/tpgp_rev.h:25-29):
// keys[k*W + w], two bits per site (I=0, X=1, Y=2, Z=3), site s in word s/32
// at bit 2*(s%32), ordered as multi-word integers with the highest word most
// significant (engine/src/tpgp_rev.c:64-72).  Kernels are templated on the
// word count W so a key lives in registers and moves with vector loads.
//
// All binary64 arithmetic uses explicitly rounded intrinsics (__dmul_rn,
// __dadd_rn) and the library is compiled with --fmad=false, so no product is
// ever contracted into an FMA: the reference's rounding model assumes
// separately rounded operations (engine/cuda/CMakeLists.txt:26-27).
#pragma once
#include <climits>
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace tg {

// ---------------------------------------------------------------- status bits
enum : unsigned {
    ST_NUMERIC = 1u,    // nonfinite branch value or merged sum -> ENUMERIC
    ST_CAPACITY = 2u,   // device buffers too small: host grows them and retries
    ST_CAP = 4u,        // active-term cap exceeded -> ECAP
    ST_BUDGET = 8u,     // drop budget exceeded -> EBUDGET
    ST_TIMEOUT = 16u,   // a bounded wait gave up -> EBACKEND
    ST_ORDER = 32u,     // input keys not strictly ascending / padding bits -> EINVAL
};

// Maximum number of map terms a device map may hold (counts are packed
// 31 bits wide in the look-back words).
constexpr unsigned long long kMaxTerms = (1ull << 30);

// -------------------------------------------------------------------- keys
template <int W>
struct Key {
    uint64_t w[W];
};

template <int W>
__device__ __forceinline__ Key<W> load_key(const uint64_t* __restrict__ keys, size_t k) {
    Key<W> r;
    if constexpr (W == 2) {
        const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(keys) + k);
        r.w[0] = v.x;
        r.w[1] = v.y;
    } else if constexpr (W == 4) {
        const ulonglong2 a = __ldg(reinterpret_cast<const ulonglong2*>(keys) + 2 * k);
        const ulonglong2 b = __ldg(reinterpret_cast<const ulonglong2*>(keys) + 2 * k + 1);
        r.w[0] = a.x;
        r.w[1] = a.y;
        r.w[2] = b.x;
        r.w[3] = b.y;
    } else {
#pragma unroll
        for (int w = 0; w < W; ++w) r.w[w] = __ldg(keys + k * W + w);
    }
    return r;
}

// Plain (coherent) load for buffers written earlier in the same kernel.
template <int W>
__device__ __forceinline__ Key<W> load_key_coherent(const uint64_t* keys, size_t k) {
    Key<W> r;
#pragma unroll
    for (int w = 0; w < W; ++w) r.w[w] = keys[k * W + w];
    return r;
}

template <int W>
__device__ __forceinline__ void store_key(uint64_t* keys, size_t k, const Key<W>& key) {
    if constexpr (W == 2) {
        reinterpret_cast<ulonglong2*>(keys)[k] = make_ulonglong2(key.w[0], key.w[1]);
    } else if constexpr (W == 4) {
        reinterpret_cast<ulonglong2*>(keys)[2 * k] = make_ulonglong2(key.w[0], key.w[1]);
        reinterpret_cast<ulonglong2*>(keys)[2 * k + 1] = make_ulonglong2(key.w[2], key.w[3]);
    } else {
#pragma unroll
        for (int w = 0; w < W; ++w) keys[k * W + w] = key.w[w];
    }
}

template <int W>
__device__ __forceinline__ bool key_eq(const Key<W>& a, const Key<W>& b) {
    bool e = true;
#pragma unroll
    for (int w = 0; w < W; ++w) e &= a.w[w] == b.w[w];
    return e;
}

// a < b as multi-word integers, highest word most significant.
template <int W>
__device__ __forceinline__ bool key_less(const Key<W>& a, const Key<W>& b) {
#pragma unroll
    for (int w = W - 1; w > 0; --w)
        if (a.w[w] != b.w[w]) return a.w[w] < b.w[w];
    return a.w[0] < b.w[0];
}

template <int W>
__device__ __forceinline__ bool key_le(const Key<W>& a, const Key<W>& b) {
    return !key_less<W>(b, a);
}

template <int W>
__device__ __forceinline__ Key<W> key_xor(const Key<W>& a, const Key<W>& m) {
    Key<W> r;
#pragma unroll
    for (int w = 0; w < W; ++w) r.w[w] = a.w[w] ^ m.w[w];
    return r;
}

template <int W>
__device__ __forceinline__ bool key_is_zero(const Key<W>& a) {
    uint64_t o = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) o |= a.w[w];
    return o == 0;
}

// Index of the highest bit where a and b differ (bit 64*w + b), -1 if equal.
template <int W>
__device__ __forceinline__ int highest_diff_bit(const Key<W>& a, const Key<W>& b) {
    int r = -1;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        const uint64_t d = a.w[w] ^ b.w[w];
        if (d) r = 64 * w + 63 - __clzll((long long)d);
    }
    return r;
}

// Word w of a key held in registers (unrolled select: no local-memory indexing).
template <int W>
__device__ __forceinline__ uint64_t word_at(const Key<W>& a, int w) {
    uint64_t r = a.w[0];
#pragma unroll
    for (int x = 1; x < W; ++x)
        if (x == w) r = a.w[x];
    return r;
}

template <int W>
__device__ __forceinline__ unsigned key_bit(const Key<W>& a, int bit) {
    return (unsigned)(word_at<W>(a, bit >> 6) >> (bit & 63)) & 1u;
}

// Element q of a small register array (unrolled select).
template <int N, typename T>
__device__ __forceinline__ T pick(const T (&v)[N], int q) {
    T r = v[0];
#pragma unroll
    for (int x = 1; x < N; ++x)
        if (x == q) r = v[x];
    return r;
}

// Keeps only bits >= theta (multi-word).
template <int W>
__device__ __forceinline__ Key<W> key_high(const Key<W>& a, int theta) {
    Key<W> r;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        const int lo = 64 * w;
        if (theta <= lo) r.w[w] = a.w[w];
        else if (theta >= lo + 64) r.w[w] = 0;
        else r.w[w] = a.w[w] & (~0ull << (theta - lo));
    }
    return r;
}

__device__ __forceinline__ unsigned site_symbol(uint64_t word, int shift) {
    return (unsigned)(word >> shift) & 3u;
}

// ---------------------------------------------------- Pauli algebra (2 sites)
// Anticommutation of single-site Paulis (engine/src/tpgp_rev.c:418).
__device__ __forceinline__ bool anticommutes(unsigned q, unsigned p) {
    return q && p && q != p;
}
// Exponent of i in Q*P (engine/src/tpgp_rev.c:414-417): +i for the cyclic
// order X->Y->Z->X, -i for the reverse, 0 when the two commute.
__device__ __forceinline__ unsigned phase_exponent(unsigned q, unsigned p) {
    if (!q || !p || q == p) return 0u;
    return ((q % 3u) + 1u == p) ? 1u : 3u;
}

// ------------------------------------------------- directed rounding helpers
// Exact successor toward +inf of a binary64 value, including zero and
// subnormal transitions (the reference's nextafter(x, INFINITY)).
__device__ __forceinline__ double next_up(double x) {
    if (x != x || x == __longlong_as_double(0x7ff0000000000000ll)) return x;
    if (x == 0.0) return __longlong_as_double(1ll);
    long long bits = __double_as_longlong(x);
    bits = x > 0 ? bits + 1 : bits - 1;
    return __longlong_as_double(bits);
}
// upadd / upmul of engine/src/tpgp_rev.c:25-36.
__device__ __forceinline__ double up_add(double a, double b) {
    if (a == 0.0) return b;
    if (b == 0.0) return a;
    return next_up(__dadd_rn(a, b));
}
__device__ __forceinline__ double up_mul(double a, double b) {
    if (a == 0.0 || b == 0.0) return 0.0;
    return next_up(__dmul_rn(a, b));
}
__device__ __forceinline__ bool is_finite(double x) {
    return (__double_as_longlong(x) & 0x7ff0000000000000ll) != 0x7ff0000000000000ll;
}

// ----------------------------------------------------------- ledger on device
// Same field order as tpgp_ledger (engine/include/tpgp_rev.h:46-51).
struct Ledger {
    double dropped_l1, dropped_l2, dropped_l2_squared, arithmetic_l2;
    unsigned long long rotations, removal_events, peak_terms;
    int arithmetic_enclosed;
};

// Device-resident state of one map's rotation sequence.
struct DeviceState {
    unsigned long long n;        // terms in the current map (input of the next rotation)
    unsigned long long a;        // anticommuting terms of the current rotation
    unsigned long long n_out;    // terms kept by the current rotation
    unsigned long long removed;  // terms removed by the threshold in the current rotation
    unsigned long long a_next;   // anticommuting terms of the next rotation (set by k_merge)
    unsigned int status;         // sticky ST_* bits
    unsigned int p1_counter, p3_counter, merge_done;
    unsigned long long p1_tiles, p3_tiles;  // tiles used (cleared by the commit kernel)
    unsigned long long rotations_done;      // rotations committed in the current call
    unsigned long long terms_in;            // input terms of the committed rotations
    Ledger ledger;
};

// --------------------------------------------------------- decoupled look-back
// One 64-bit word per tile: [flag:2 | hi:31 | lo:31].  flag 1 = tile
// aggregate published, 2 = inclusive prefix published.  Words are cleared
// by the commit kernel after every rotation.
constexpr unsigned long long kFlagAgg = 1ull << 62, kFlagPre = 2ull << 62;
constexpr unsigned long long kCountMask = (1ull << 31) - 1;
// A look-back wait gives up after this many polls (~0.1-1 s) and reports
// ST_TIMEOUT instead of spinning forever.
constexpr unsigned kLookbackPolls = 1u << 22;

__device__ __forceinline__ unsigned long long pack2(unsigned long long lo, unsigned long long hi) {
    return (lo & kCountMask) | ((hi & kCountMask) << 31);
}
__device__ __forceinline__ void unpack2(unsigned long long v, unsigned long long& lo,
                                        unsigned long long& hi) {
    lo = v & kCountMask;
    hi = (v >> 31) & kCountMask;
}

__device__ __forceinline__ void publish(unsigned long long* slot, unsigned long long word) {
    __threadfence();
    atomicExch(slot, word);
}
__device__ __forceinline__ unsigned long long poll(const unsigned long long* slot) {
    return *reinterpret_cast<const volatile unsigned long long*>(slot);
}

// Called by warp 0 of the block that owns `tile`; returns the exclusive
// prefix (two packed counters) of all earlier tiles.  Publishes this tile's
// aggregate first, then its inclusive prefix.
__device__ inline unsigned long long lookback_exclusive(unsigned long long* tiles,
                                                        unsigned long long tile,
                                                        unsigned long long agg_packed,
                                                        unsigned int* status) {
    const unsigned lane = threadIdx.x & 31;
    if (tile == 0) {
        if (lane == 0) publish(tiles, kFlagPre | agg_packed);
        return 0;
    }
    if (lane == 0) publish(tiles + tile, kFlagAgg | agg_packed);
    unsigned long long lo = 0, hi = 0;
    long long base = (long long)tile - 1;
    bool done = false;
    unsigned polls = 0;
    while (!done) {
        // each lane inspects one predecessor: base - lane
        const long long t = base - (long long)lane;
        unsigned long long word = kFlagPre;  // below tile 0: an empty prefix
        if (t >= 0) {
            word = poll(tiles + t);
            while ((word >> 62) == 0) {
                if (++polls > kLookbackPolls) {
                    atomicOr(status, ST_TIMEOUT);
                    word = kFlagPre;  // give up: treat as an empty prefix
                    break;
                }
                word = poll(tiles + t);
            }
        }
        const unsigned pre_mask = __ballot_sync(0xffffffffu, (word >> 62) == 2);
        // lanes up to (and including) the first inclusive prefix contribute
        const unsigned first_pre = pre_mask ? (unsigned)__ffs(pre_mask) - 1 : 32u;
        unsigned long long l = 0, h = 0;
        if (lane <= first_pre && lane < 32) unpack2(word, l, h);
        if (lane > first_pre) { l = 0; h = 0; }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            l += __shfl_down_sync(0xffffffffu, l, off);
            h += __shfl_down_sync(0xffffffffu, h, off);
        }
        lo += __shfl_sync(0xffffffffu, l, 0);
        hi += __shfl_sync(0xffffffffu, h, 0);
        if (pre_mask) done = true;
        base -= 32;
    }
    if (lane == 0) {
        unsigned long long al, ah;
        unpack2(agg_packed, al, ah);
        publish(tiles + tile, kFlagPre | pack2(lo + al, hi + ah));
    }
    return pack2(lo, hi);
}

}  // namespace tg
