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

// ------------------------------------------------ programmatic dependent launch
// A kernel launched with programmatic stream serialization may be scheduled
// while its predecessor on the stream is still running.  It waits here for
// the predecessor's completion (and the visibility of its memory) before it
// touches any state, then lets its own successor be scheduled, so only the
// launch latency overlaps, never the work.  Launched without the attribute,
// both instructions return at once.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// ------------------------------------------------------------------ lanes
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---------------------------------------------------------------- status bits
enum : unsigned {
    ST_NUMERIC = 1u,    // nonfinite branch value or merged sum -> ENUMERIC
    ST_CAPACITY = 2u,   // device buffers too small: host grows them and retries
    ST_CAP = 4u,        // active-term cap exceeded -> ECAP
    ST_BUDGET = 8u,     // drop budget exceeded -> EBUDGET
    ST_TIMEOUT = 16u,   // a bounded wait gave up -> EBACKEND
    ST_ORDER = 32u,     // input keys not strictly ascending / padding bits -> EINVAL
    ST_TABLE = 64u,     // hash-table step: probe bound hit; host enlarges the table and retries
    ST_LOG = 128u,      // exact-ledger log of removed values too small: host enlarges it and retries
};

// Maximum number of map terms a device map may hold (counts are packed
// 31 bits wide in the look-back words).
constexpr unsigned long long kMaxTerms = (1ull << 30);

// -------------------------------------------------------------------- keys
template <int W>
struct Key {
    uint64_t w[W];
};

// Loads of kernel data use ld.global.cg (L2, not the L1 or read-only
// caches): the persistent step kernel reads, after a grid barrier, buffers
// that other SMs wrote earlier in the same launch, where an L1 or
// non-coherent cached copy could be stale.
template <int W>
__device__ __forceinline__ Key<W> load_key(const uint64_t* keys, size_t k) {
    Key<W> r;
    if constexpr (W == 2) {
        const ulonglong2 v = __ldcg(reinterpret_cast<const ulonglong2*>(keys) + k);
        r.w[0] = v.x;
        r.w[1] = v.y;
    } else if constexpr (W == 4) {
        const ulonglong2 a = __ldcg(reinterpret_cast<const ulonglong2*>(keys) + 2 * k);
        const ulonglong2 b = __ldcg(reinterpret_cast<const ulonglong2*>(keys) + 2 * k + 1);
        r.w[0] = a.x;
        r.w[1] = a.y;
        r.w[2] = b.x;
        r.w[3] = b.y;
    } else {
#pragma unroll
        for (int w = 0; w < W; ++w) r.w[w] = __ldcg(keys + k * W + w);
    }
    return r;
}

template <int W>
__device__ __forceinline__ Key<W> load_key_coherent(const uint64_t* keys, size_t k) {
    return load_key<W>(keys, k);
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
// GB300 issues binary64 arithmetic at a small fraction of its integer rate,
// so every exact predicate on a binary64 value (zero test, absolute value,
// sign flip, comparison of non-negative values, successor) works on the bit
// pattern with integer instructions; only genuine products and sums use the
// FP64 pipe.  For non-negative finite doubles the IEEE order equals the
// unsigned order of their bit patterns.
constexpr unsigned long long kSignBit = 0x8000000000000000ull;
constexpr unsigned long long kExpMask = 0x7ff0000000000000ull;

// Register moves the compiler cannot see through, so that sign, absolute
// value and zero tests on the bit pattern stay integer instructions instead
// of being folded back into FP64 negate/abs/compare operations.
__device__ __forceinline__ unsigned long long dbits(double x) {
    unsigned long long u;
    asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
    return u;
}
__device__ __forceinline__ double from_bits(unsigned long long u) {
    double x;
    asm("mov.b64 %0, %1;" : "=d"(x) : "l"(u));
    return x;
}
__device__ __forceinline__ bool is_zero(double x) { return (dbits(x) << 1) == 0; }
__device__ __forceinline__ bool is_finite(double x) { return (dbits(x) & kExpMask) != kExpMask; }
__device__ __forceinline__ unsigned long long abs_bits(double x) { return dbits(x) & ~kSignBit; }
__device__ __forceinline__ double abs_of(double x) { return from_bits(abs_bits(x)); }
__device__ __forceinline__ double negate(double x) { return from_bits(dbits(x) ^ kSignBit); }

// Exact successor toward +inf (the reference's nextafter(x, INFINITY)),
// including zero and subnormal transitions; NaN and +inf are unchanged.
__device__ __forceinline__ double next_up(double x) {
    const unsigned long long u = dbits(x);
    if ((u << 1) == 0) return from_bits(1ull);             // +-0 -> smallest subnormal
    if ((u & ~kSignBit) > kExpMask || u == kExpMask) return x;  // NaN, +inf
    return from_bits((u & kSignBit) ? u - 1 : u + 1);
}
// upadd / upmul of engine/src/tpgp_rev.c:25-36.
__device__ __forceinline__ double up_add(double a, double b) {
    if (is_zero(a)) return b;
    if (is_zero(b)) return a;
    return next_up(__dadd_rn(a, b));
}
__device__ __forceinline__ double up_mul(double a, double b) {
    if (is_zero(a) || is_zero(b)) return 0.0;
    return next_up(__dmul_rn(a, b));
}

// Largest |x - neighbour| over the two adjacent binary64 values, +inf for a
// nonfinite x: round_radius of engine/src/tpgp_rev.c:37-42.
__device__ __forceinline__ double rounding_radius(double x) {
    if (!is_finite(x)) return from_bits(kExpMask);
    const double up = next_up(x), down = negate(next_up(negate(x)));
    const double a = abs_of(__dsub_rn(up, x)), b = abs_of(__dsub_rn(x, down));
    return a > b ? a : b;
}

// A chain of up_add over the lanes' addends, in lane order, computed by the
// warp together with the same result bits as the sequential chain:
// returns up_add(...up_add(up_add(s, x_0), x_1)..., x_31) over the lanes
// with `has` (warp-uniform s in, warp-uniform result out) and sets *mine to
// the chain's value after this lane's addend.  Every lane of the warp calls.
//
// While s stays in one binade [2^(E-1023), 2^(E-1022)) (E its biased
// exponent, E >= 1) its values are the integers bits(s) + k on a grid of ulp
// 2^(E-1075).  An addend x >= 0 whose exponent is at most E adds
// round(x / ulp) grid steps when s + x stays in the binade (round to
// nearest; an exact half is a tie whose direction depends on s's last bit),
// and next_up adds one more.  So each lane's step count is known without the
// chain, an inclusive warp scan of the counts gives every lane's result as
// bits, and the scan is valid up to the first lane whose result would leave
// the binade, whose addend is a tie, larger than s's binade, zero-exponent s,
// or not finite: that lane's step is taken with up_add itself, and the scan
// resumes after it with the new s.  A zero addend is no step (up_add(s, 0) = s).
__device__ __forceinline__ double warp_up_sum(double s, double x, bool has, double* mine) {
    constexpr unsigned long long kMant = (1ull << 52) - 1;
    const unsigned lane = threadIdx.x & 31u;
    unsigned start = 0;
    double my = s;
    for (;;) {
        const unsigned long long sb = dbits(s);
        const unsigned long long E = sb >> 52;  // >= 2047 for a negative or nonfinite s
        const bool pend = has && lane >= start;
        unsigned long long inc = 0;
        bool flag = false;
        if (pend && !is_zero(x)) {
            const unsigned long long xb = dbits(x);
            const unsigned long long Ex = xb >> 52;
            if (E == 0 || E >= 2047 || Ex >= 2047) {
                flag = true;
            } else {
                const unsigned long long Mx = (xb & kMant) | (Ex ? (1ull << 52) : 0ull);
                const unsigned long long Exe = Ex ? Ex : 1ull;  // subnormal x: exponent 1, no implicit bit
                if (Exe > E) {
                    flag = true;
                } else {
                    const unsigned long long d = E - Exe;
                    unsigned long long q = 0;
                    if (d == 0) {
                        q = Mx;
                    } else if (d < 64) {
                        q = Mx >> d;
                        const unsigned long long rem = Mx & ((1ull << d) - 1), half = 1ull << (d - 1);
                        if (rem > half) ++q;
                        else if (rem == half) flag = true;
                    }
                    inc = q + 1;
                }
            }
        }
        unsigned long long S = inc;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, S, off);
            if (lane >= (unsigned)off) S += y;
        }
        const unsigned long long B = (E + 1) << 52;
        const bool bad = pend && (flag || sb + S >= B);
        const unsigned m = __ballot_sync(0xffffffffu, bad);
        const unsigned L = m ? (unsigned)(__ffs(m) - 1) : 32u;
        if (lane >= start && lane < L) my = from_bits(sb + S);
        if (!m) {
            s = from_bits(sb + __shfl_sync(0xffffffffu, S, 31));
            break;
        }
        const unsigned long long before = sb + __shfl_sync(0xffffffffu, S - inc, L);
        const double xl = __shfl_sync(0xffffffffu, x, L);
        s = up_add(from_bits(before), xl);
        if (lane == L) my = s;
        start = L + 1;
        if (start >= 32) break;
    }
    if (mine) *mine = my;
    return s;
}

// ------------------------------------------------- fixed-point ledger sums
// Upper bounds on sums of removed |v| and v^2 in 128-bit integer fixed
// point: each addend is rounded UP to a multiple of 2^unit, the sum is exact
// (order-independent), and the total is converted to binary64 rounding up.
// The unit is chosen from the threshold t (removed |v| <= t < 2^et):
// unit1 = et - 96, unit2 = 2 et - 96, so fewer than 2^31 addends never
// overflow 127 bits.
struct U128 {
    unsigned long long lo, hi;
};
__device__ __forceinline__ void u128_add(U128& a, const U128& b) {
    const unsigned long long lo = a.lo + b.lo;
    a.hi += b.hi + (lo < a.lo ? 1ull : 0ull);
    a.lo = lo;
}
// ceil(x / 2^q) for a 128-bit x and 0 <= q
__device__ __forceinline__ U128 u128_shr_ceil(U128 x, int q) {
    if (q <= 0) return x;
    if (q >= 128) return U128{(x.lo | x.hi) ? 1ull : 0ull, 0ull};
    U128 r;
    unsigned long long lost;
    if (q >= 64) {
        lost = x.lo | (q > 64 ? (x.hi << (128 - q)) : 0ull);
        r.lo = q == 64 ? x.hi : (x.hi >> (q - 64));
        r.hi = 0;
    } else {
        lost = x.lo << (64 - q);
        r.lo = (x.lo >> q) | (x.hi << (64 - q));
        r.hi = x.hi >> q;
    }
    if (lost) {
        const U128 one{1ull, 0ull};
        u128_add(r, one);
    }
    return r;
}
// m * 2^eb with m the 53-bit significand of |v| (binary64, finite, nonzero)
__device__ __forceinline__ void split_abs(double v, unsigned long long& m, int& eb) {
    const unsigned long long a = abs_bits(v);
    const int be = (int)(a >> 52);
    m = (a & 0x000fffffffffffffull) | (be ? 0x0010000000000000ull : 0ull);
    eb = (be ? be : 1) - 1075;
}
// ceil(|v| / 2^unit1) and ceil(v^2 / 2^unit2); requires |v| < 2^et
__device__ __forceinline__ void fixed_terms(double v, int unit1, int unit2, U128& x1, U128& x2) {
    unsigned long long m;
    int eb;
    split_abs(v, m, eb);
    const int sh = eb - unit1;  // <= 43 because |v| < 2^(unit1 + 96)
    if (sh >= 0) {
        x1.lo = sh == 0 ? m : (m << sh);
        x1.hi = sh == 0 ? 0ull : (sh >= 64 ? 0ull : (m >> (64 - sh)));
    } else {
        x1 = u128_shr_ceil(U128{m, 0ull}, -sh);
    }
    const U128 sq{m * m, __umul64hi(m, m)};
    x2 = u128_shr_ceil(sq, unit2 - 2 * eb);  // shift >= 10
}
__device__ __forceinline__ U128 shfl_down_u128(const U128& x, int off) {
    return U128{__shfl_down_sync(0xffffffffu, x.lo, off), __shfl_down_sync(0xffffffffu, x.hi, off)};
}
// x * 2^unit rounded up to binary64 (one FP64 scaling per rotation)
__device__ inline double u128_to_double_up(U128 x, int unit) {
    if (!(x.lo | x.hi)) return 0.0;
    const int nb = x.hi ? 128 - __clzll((long long)x.hi) : 64 - __clzll((long long)x.lo);
    int shift = nb > 53 ? nb - 53 : 0;
    U128 t = u128_shr_ceil(x, shift);
    if (t.lo >> 53) {  // rounding carried to 2^53
        t.lo >>= 1;
        ++shift;
    }
    const double r = ldexp((double)t.lo, unit + shift);
    return r;
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
    unsigned int bar_count, bar_gen;  // grid barrier of the persistent kernel
    unsigned int stop;                // set by the committing CTA when the rotation failed
    unsigned long long p1_tiles, p3_tiles;  // tiles used (cleared by the commit kernel)
    unsigned long long rotations_done;      // rotations committed in the current call
    unsigned long long terms_in;            // input terms of the committed rotations
    Ledger ledger;
    // the hash-table step's input and output map buffers, set per call, so
    // one captured step serves whichever buffers hold the map
    const uint64_t* in_keys;
    const double* in_vals;
    uint64_t* out_keys;
    double* out_vals;
    unsigned long long out_cap;
    // exact ledger: next free position of the call's log of removed |v|, and
    // the size a retry needs when the log ran out
    unsigned long long log_pos, log_need;
    // poll limit of every device-side wait of the call (0: the defaults), and
    // extra arrivals a grid barrier waits for (nonzero only to test that a
    // wait which can never end gives up: a participant that does not exist)
    unsigned wait_polls, bar_extra;
};

__device__ __forceinline__ unsigned poll_limit(const DeviceState* st, unsigned dflt) {
    const unsigned v = *reinterpret_cast<const volatile unsigned*>(&st->wait_polls);
    return v ? v : dflt;
}

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
                                                        unsigned int* status,
                                                        unsigned limit = kLookbackPolls) {
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
                if (++polls > limit) {
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
