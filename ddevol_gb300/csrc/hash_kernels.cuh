// Sort-free Strang step for the bound ledger: the map lives in an
// open-addressing hash table for the duration of one step, every rotation is
// one pass over the table's occupied slots, and the map is sorted back into
// the reference layout once per step.
//
// Why it is exact.  A rotation by Q pairs every anticommuting key K with its
// partner K xor Q (anticommutation with Q is invariant under multiplication
// by Q), and the reference's merged value of K is RN(RN(v_K c) + s_P RN(v_P s))
// when both are in the map, RN(v_K c) or s_P RN(v_P s) when only one is
// (engine/src/tpgp_rev.c:420-467 branch, :693-729 merge; s_P is the phase
// sign of the partner's child).  Each pair is therefore updated on its own:
// one thread computes both new values with those exact operations, drops
// exact zeros, applies the threshold (identity key exempt; commuting keys
// keep v + 0 = v but are thresholded like every merged term) and accumulates
// the removed |v| and v^2 into the same 128-bit fixed-point sums the sorted
// path uses, so keys, values and the bound ledger are bitwise those of the
// sorted path.
//
// Table.  One record per slot -- the key, the value's bit pattern and a tag
// (0 empty, 1 present at step start, k+2 inserted by pass k) -- 32 bytes for
// one- and two-word keys (a single 32-byte load), 48 bytes for three and four
// words.  Keys never leave the table during a step (a removed key keeps its
// slot with value 0), so linear probing needs no tombstones: a present key is
// always found before the first empty slot of its probe sequence.  Every
// claimed slot is also appended to an occupied-slot list in claim order, and
// a pass walks that list, so its threads see only occupied slots (whatever
// the table's load) and a warp's lanes do the same kind of work.
//
// Values are updated in place.  The pair {K, K xor Q} is owned by its
// smaller member among the keys present when the pass starts (dead keys,
// value 0, included); ownership depends on keys and tags only, which no
// thread changes during a pass, so exactly one thread reads and writes the
// pair's two values, and a commuting key's value is touched by its own
// thread only.  A dead member contributes no child: the owner combines the
// live members exactly as the reference merges the children that exist.  A
// key looked up in pass k is never inserted by another thread in k (only its
// pair's owner inserts it), so probes skip slots tagged k+2.
//
// Ledger and limits.  Each rotation adds its born/died/removed counts and
// fixed-point sums to per-rotation stat slots; k_hash_chain then applies,
// rotation by rotation on one thread, exactly the commit of
// engine/src/tpgp_rev.c:730-757 (ECAP, ledger, ENUMERIC, EBUDGET), stopping
// at the first failure.  Work after a failing rotation is discarded: the
// step's input map is never written (transactional).
#pragma once
#include <cooperative_groups.h>

#include "onesweep.cuh"
#include "rotate_kernels.cuh"

namespace tg {

constexpr int kHashBlock = 256;
constexpr int kMaxProbe = 2048;  // linear-probe bound; hitting it reports ST_TABLE
constexpr int kStatSlots = 32;   // stat slots per rotation (spreads the atomics)
constexpr uint32_t kNoSlot = 0xffffffffu;  // list entry reserved but not yet written

// Per-rotation stat slot.  The removed-weight sums are 128-bit integers
// accumulated as four 32-bit limbs, each summed in its own 64-bit counter by
// reductions that return nothing (no CTA waits on an atomic's result);
// k_hash_reduce recombines the limbs exactly (fewer than 2^32 addends per
// counter).
struct HashStat {
    unsigned long long l1[4], sq[4];
    unsigned long long born, died, removed;
    unsigned int flags, pad;
    unsigned long long radii;  // merged radii logged (validated rotations)
    unsigned long long unused[3];
};
static_assert(sizeof(HashStat) == 128, "stat slot is two 64-byte lines");

// What a pass needs of its rotation, passed by value as a kernel parameter
// (constant bank) so no thread waits on a global load for it.
// anti / plus: bit 4 pi + pj is set when a key with symbols (pi, pj) at the
// rotation's sites anticommutes with the generator / has a + sign on its
// sin child (the phase table of engine/src/tpgp_rev.c:414-417); the
// partner's index is the key's xor qmix = 4 qi + qj.
// settled: 1 when every live value already passed this pass's threshold (a
// later pass of a list with one threshold), so commuting keys, whose value
// the rotation leaves unchanged, need no work at all.
struct PassParams {
    int i_word, i_shift, j_word, j_shift;
    unsigned qi, qj;
    unsigned anti, plus, qmix;
    unsigned settled;
    double c, s;
    unsigned long long threshold_bits;
    uint64_t mask[4];
    int fx_unit1, fx_unit2;
    unsigned validated;  // children carry error radii (rc, rs)
    double rc, rs;
};

__host__ __device__ inline PassParams pass_params(const RotParams& r) {
    PassParams p;
    p.i_word = r.i_word;
    p.i_shift = r.i_shift;
    p.j_word = r.j_word;
    p.j_shift = r.j_shift;
    p.qi = r.qi;
    p.qj = r.qj;
    p.anti = p.plus = 0u;
    for (unsigned pi = 0; pi < 4; ++pi)
        for (unsigned pj = 0; pj < 4; ++pj) {
            const bool ai = r.qi && pi && r.qi != pi, aj = r.qj && pj && r.qj != pj;
            const unsigned ei = ai ? ((r.qi % 3u) + 1u == pi ? 1u : 3u) : 0u;
            const unsigned ej = aj ? ((r.qj % 3u) + 1u == pj ? 1u : 3u) : 0u;
            if (ai != aj) p.anti |= 1u << (4 * pi + pj);
            if (((ei + ej) & 3u) == 1u) p.plus |= 1u << (4 * pi + pj);
        }
    p.qmix = 4u * r.qi + r.qj;
    p.settled = 0u;
    p.c = r.c;
    p.s = r.s;
    p.threshold_bits = r.threshold_bits;
    for (int w = 0; w < 4; ++w) p.mask[w] = r.mask[w];
    p.fx_unit1 = r.fx_unit1;
    p.fx_unit2 = r.fx_unit2;
    p.validated = r.validated ? 1u : 0u;
    p.rc = r.rc;
    p.rs = r.rs;
    return p;
}

struct HashArgs {
    const RotParams* ps;  // the step's rotation list (device)
    unsigned rotations;
    const uint2* runs;    // fused passes: (first rotation, count) per pass
    unsigned passes;      // kernels over the table (= rotations when not fused)
    unsigned long long* rec;        // [S] records of rec_words<W>() words
    unsigned long long* occ;        // occupied-slot list: entries of list_words<W>() words
    unsigned long long slots;       // S (any size: slots are h * S >> 64)
    HashStat* stats;                // [rotations][kStatSlots]
    unsigned long long* claimed;    // slots claimed during the step = entries of occ
    uint64_t* ek;                   // extraction / sort ping-pong buffers, S entries
    unsigned long long* ev;
    uint64_t* tk;
    unsigned long long* tv;
    DeviceState* st;
    // exact ledger: every removed term's key (W words) and |v| bits.  The
    // passes of a step run in rotation order, so each rotation's entries form
    // one contiguous segment of the log (in any order within it), of the
    // length its stat slots count as removed.  xlog_keys == nullptr: bound ledger.
    uint64_t* xlog_keys;
    unsigned long long* xlog_vals;
    unsigned long long xlog_cap;
    unsigned long long* xlog_count;
};

// Appends an entry to the exact ledger's log: a removed term's |v| bits, or
// (sign bit set) a validated rotation's merged radius of the key.
template <int W>
__device__ __forceinline__ void log_entry(const HashArgs& a, const Key<W>& key,
                                          unsigned long long bits) {
    // one counter for the whole step: the threads that log together take
    // their positions with one atomic
    const cooperative_groups::coalesced_group g = cooperative_groups::coalesced_threads();
    unsigned long long pos = 0;
    if (g.thread_rank() == 0) pos = atomicAdd(a.xlog_count, (unsigned long long)g.size());
    pos = g.shfl(pos, 0) + g.thread_rank();
    if (pos >= a.xlog_cap) return;  // counted: the step reports the log full
    store_key<W>(a.xlog_keys, pos, key);
    a.xlog_vals[pos] = bits;
}
template <int W>
__device__ __forceinline__ void log_removed(const HashArgs& a, const Key<W>& key, double x) {
    log_entry<W>(a, key, abs_bits(x));
}


// Record layout: words 0..W-1 the key, word W the value bits, the low half
// of word W+1 the tag.
template <int W>
__host__ __device__ constexpr int rec_words() {
    return W <= 2 ? 4 : 6;
}

template <int W>
struct Rec {
    Key<W> key;
    unsigned long long val;
    uint32_t tag;
};

// One record in one access for W <= 2 (a 32-byte vector load, L2 only: the
// persistent variant reads records other SMs wrote in the same launch).
template <int W>
__device__ __forceinline__ Rec<W> load_rec(const unsigned long long* rec, unsigned long long s) {
    const unsigned long long* p = rec + s * rec_words<W>();
    Rec<W> r;
    if constexpr (W <= 2) {
        unsigned long long x0, x1, x2, x3;
        asm volatile("ld.global.cg.v4.u64 {%0, %1, %2, %3}, [%4];"
                     : "=l"(x0), "=l"(x1), "=l"(x2), "=l"(x3)
                     : "l"(p));
        r.key.w[0] = x0;
        if constexpr (W == 1) {
            r.val = x1;
            r.tag = (uint32_t)x2;
        } else {
            r.key.w[1] = x1;
            r.val = x2;
            r.tag = (uint32_t)x3;
        }
    } else {
        const ulonglong2 a = __ldcg(reinterpret_cast<const ulonglong2*>(p));
        const ulonglong2 b = __ldcg(reinterpret_cast<const ulonglong2*>(p) + 1);
        const ulonglong2 c = __ldcg(reinterpret_cast<const ulonglong2*>(p) + 2);
        const unsigned long long x[6] = {a.x, a.y, b.x, b.y, c.x, c.y};
#pragma unroll
        for (int w = 0; w < W; ++w) r.key.w[w] = x[w];
        r.val = x[W];
        r.tag = (uint32_t)x[W + 1];
    }
    return r;
}

template <int W>
__device__ __forceinline__ uint32_t* rec_tag(unsigned long long* rec, unsigned long long s) {
    return reinterpret_cast<uint32_t*>(rec + s * rec_words<W>() + W + 1);
}
template <int W>
__device__ __forceinline__ void store_val(unsigned long long* rec, unsigned long long s,
                                          unsigned long long bits) {
    rec[s * rec_words<W>() + W] = bits;
}

__device__ __forceinline__ unsigned long long fmix64(unsigned long long h) {
    h ^= h >> 33;
    h *= 0xff51afd7ed558ccdull;
    h ^= h >> 33;
    h *= 0xc4ceb9fe1a85ec53ull;
    h ^= h >> 33;
    return h;
}
// Hash of a key: the words folded through the murmur3 64-bit finalizer.
// (A plain multiplicative hash was tried: its low bits cluster on Pauli
// keys, whose nonidentity sites are few, and probe chains grew ~20x.)
template <int W>
__device__ __forceinline__ unsigned long long hash_of(const Key<W>& k) {
    unsigned long long h = 0x9e3779b97f4a7c15ull;
#pragma unroll
    for (int w = 0; w < W; ++w) h = fmix64(h ^ k.w[w]);
    return h;
}

// Table slot of a hash (the high word of h * S: uniform over any S) and the
// next slot of a linear probe.
__device__ __forceinline__ unsigned long long slot_of(unsigned long long h, unsigned long long S) {
    return __umul64hi(h, S);
}
__device__ __forceinline__ unsigned long long next_slot(unsigned long long s, unsigned long long S) {
    return s + 1 == S ? 0ull : s + 1;
}

// Branch data of key K and of its partner K xor Q from K's two site symbols
// (the partner's symbols are K's xor (qi, qj)).
__device__ __forceinline__ void pair_signs(const RotParams& p, uint64_t wi, uint64_t wj,
                                           bool& anti, bool& plus_k, bool& plus_p) {
    const unsigned pi = site_symbol(wi, p.i_shift), pj = site_symbol(wj, p.j_shift);
    anti = anticommutes(p.qi, pi) != anticommutes(p.qj, pj);
    plus_k = ((phase_exponent(p.qi, pi) + phase_exponent(p.qj, pj)) & 3u) == 1u;
    plus_p = ((phase_exponent(p.qi, pi ^ p.qi) + phase_exponent(p.qj, pj ^ p.qj)) & 3u) == 1u;
}

// Looks up key k from its first probe slot `s`, whose record `r` the caller
// has already loaded: returns its slot (tags equal to `skip` ignored), or -1
// with *empty_at the first empty slot of the probe sequence; *overflow when
// the probe bound is hit.  *rv receives the found record's value.
template <int W>
__device__ __forceinline__ long long probe_from(const HashArgs& a, const Key<W>& k,
                                                unsigned long long s, Rec<W> r, uint32_t skip,
                                                unsigned long long* empty_at,
                                                unsigned long long* rv, bool* overflow) {
    for (int i = 0; i < kMaxProbe; ++i) {
        if (r.tag == 0u) {
            *empty_at = s;
            return -1;
        }
        if (r.tag != skip && key_eq<W>(r.key, k)) {
            *rv = r.val;
            return (long long)s;
        }
        s = next_slot(s, a.slots);
        r = load_rec<W>(a.rec, s);
    }
    *overflow = true;
    return -1;
}

// Claims the first empty slot at or after `from` for k (tag `stamp`) and
// writes its key and value; the caller appends the slot to the list.
template <int W>
__device__ __forceinline__ long long hash_insert(const HashArgs& a, const Key<W>& k,
                                                 unsigned long long bits, unsigned long long from,
                                                 uint32_t stamp, bool* overflow) {
    unsigned long long s = from;
    for (int i = 0; i < kMaxProbe; ++i) {
        uint32_t* tag = rec_tag<W>(a.rec, s);
        if (__ldcg(tag) == 0u && atomicCAS(tag, 0u, stamp) == 0u) {
            unsigned long long* p = a.rec + s * rec_words<W>();
#pragma unroll
            for (int w = 0; w < W; ++w) p[w] = k.w[w];
            p[W] = bits;
            return (long long)s;
        }
        s = next_slot(s, a.slots);
    }
    *overflow = true;
    return -1;
}

// Occupied-slot list entry: the key (words 0..W-1; keys never change during
// a step, so a pass reads a key here and starts its partner probe without
// first loading the slot's record) and, in word W, the slot (low half) and
// the stamp of the pass that claimed it (high half), stored together so a
// reader never sees one without the other.  An entry whose word W is all
// ones (the list's fill) is reserved but not yet written.
template <int W>
__host__ __device__ constexpr int list_words() {
    return W == 1 ? 2 : (W <= 3 ? 4 : 6);
}
constexpr unsigned long long kNoEntry = ~0ull;

template <int W>
struct Entry {
    Key<W> key;
    uint32_t slot, stamp;  // slot kNoSlot: not written yet
};

template <int W>
__device__ __forceinline__ Entry<W> load_entry(const unsigned long long* occ, unsigned long long i) {
    const unsigned long long* p = occ + i * list_words<W>();
    Entry<W> e;
    unsigned long long tail;
    if constexpr (W == 1) {
        const ulonglong2 v = __ldcg(reinterpret_cast<const ulonglong2*>(p));
        e.key.w[0] = v.x;
        tail = v.y;
    } else if constexpr (W <= 3) {
        unsigned long long x0, x1, x2, x3;
        asm volatile("ld.global.cg.v4.u64 {%0, %1, %2, %3}, [%4];"
                     : "=l"(x0), "=l"(x1), "=l"(x2), "=l"(x3)
                     : "l"(p));
        const unsigned long long x[4] = {x0, x1, x2, x3};
#pragma unroll
        for (int w = 0; w < W; ++w) e.key.w[w] = x[w];
        tail = x[W];
    } else {
        const ulonglong2 a = __ldcg(reinterpret_cast<const ulonglong2*>(p));
        const ulonglong2 b = __ldcg(reinterpret_cast<const ulonglong2*>(p) + 1);
        const ulonglong2 c = __ldcg(reinterpret_cast<const ulonglong2*>(p) + 2);
        e.key.w[0] = a.x;
        e.key.w[1] = a.y;
        e.key.w[2] = b.x;
        e.key.w[3] = b.y;
        tail = c.x;
    }
    e.slot = tail == kNoEntry ? kNoSlot : (uint32_t)tail;
    e.stamp = (uint32_t)(tail >> 32);
    return e;
}

template <int W>
__device__ __forceinline__ void store_entry(unsigned long long* occ, unsigned long long i,
                                            const Key<W>& k, unsigned long long slot, uint32_t stamp) {
    unsigned long long* p = occ + i * list_words<W>();
#pragma unroll
    for (int w = 0; w < W; ++w) p[w] = k.w[w];
    p[W] = (slot & 0xffffffffull) | ((unsigned long long)stamp << 32);
}

// Reserves list entries for the lanes with `want` set (one atomic per warp;
// every lane of the warp calls it) and returns each such lane's index.
__device__ __forceinline__ unsigned long long list_reserve(const HashArgs& a, bool want) {
    const unsigned m = __ballot_sync(0xffffffffu, want);
    if (!m) return 0ull;
    const unsigned lane = threadIdx.x & 31u, leader = (unsigned)(__ffs(m) - 1);
    unsigned long long at = 0;
    if (lane == leader) at = atomicAdd(a.claimed, (unsigned long long)__popc(m));
    at = __shfl_sync(0xffffffffu, at, leader);
    return at + __popc(m & lanemask_lt());
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long x) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
    return x;
}

// Adds a 128-bit value into a (lo, hi) pair of counters, exactly, under
// concurrent adders: the carry of each lo addition follows from the old value.
__device__ __forceinline__ void atomic_add_u128(unsigned long long* lo, unsigned long long* hi,
                                                const U128& x) {
    unsigned long long carry = 0;
    if (x.lo) {
        const unsigned long long old = atomicAdd(lo, x.lo);
        carry = old + x.lo < old ? 1ull : 0ull;
    }
    if (x.hi + carry) atomicAdd(hi, x.hi + carry);
}

// --------------------------------------------------------------- build
// Inserts the step's input map (stamp 1).  Loops are warp-uniform so that
// list_reserve's ballot sees every lane.
template <int W>
__global__ void __launch_bounds__(kHashBlock) k_hash_build(HashArgs a) {
    bool overflow = false;
    const unsigned long long n = __ldcg(&a.st->n);
    // the step's input map (never written)
    const uint64_t* in_keys = a.st->in_keys;
    const double* in_vals = a.st->in_vals;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u);
         base < n; base += stride) {
        const unsigned long long k = base + lane;
        long long s = -1;
        Key<W> key;
        if (k < n) {
            key = load_key<W>(in_keys, k);
            const unsigned long long bits = dbits(__ldcg(in_vals + k));
            s = hash_insert<W>(a, key, bits, slot_of(hash_of<W>(key), a.slots), 1u, &overflow);
        }
        const unsigned long long at = list_reserve(a, s >= 0);
        if (s >= 0) store_entry<W>(a.occ, at, key, (unsigned long long)s, 1u);
    }
    if (overflow) atomicOr(&a.st->status, ST_TABLE);
}

// --------------------------------------------------------------- rotation
// Per-thread counts (32-bit: a thread handles far fewer than 2^32 slots)
// and removed-weight sums (exact 128-bit fixed point), reduced per warp by
// shuffles and per CTA once at the end of a pass, so no thread waits on a
// shared or global atomic while it removes terms.
struct PairTally {
    unsigned born, died, removed, flags;
    unsigned radii;
    U128 l1, sq;
};

__device__ __forceinline__ PairTally empty_tally() {
    PairTally t;
    t.born = t.died = t.removed = t.flags = t.radii = 0u;
    t.l1 = U128{0ull, 0ull};
    t.sq = U128{0ull, 0ull};
    return t;
}

// Exact 128-bit accumulation into shared memory under concurrent adders.
__device__ __forceinline__ void shared_add_u128(unsigned long long* acc, const U128& x) {
    unsigned long long carry = 0;
    if (x.lo) {
        const unsigned long long old = atomicAdd(acc, x.lo);
        carry = old + x.lo < old ? 1ull : 0ull;
    }
    if (x.hi + carry) atomicAdd(acc + 1, x.hi + carry);
}

// New value of one key of a pair: exact zero -> dropped; |x| <= threshold
// (identity exempt) -> removed into the fixed-point sums; else kept.
// Returns the bit pattern to store (0 when dropped or removed).
template <int W, typename P>
__device__ __forceinline__ unsigned long long settle(const P& p, const Key<W>& key,
                                                     double x, bool was_live, PairTally& t) {
    if (!is_finite(x)) t.flags |= ST_NUMERIC;
    unsigned long long out = dbits(x);
    if (is_zero(x)) {
        out = 0;
    } else if (!key_is_zero<W>(key) && abs_bits(x) <= p.threshold_bits) {
        U128 x1, x2;
        fixed_terms(x, p.fx_unit1, p.fx_unit2, x1, x2);
        u128_add(t.l1, x1);
        u128_add(t.sq, x2);
        ++t.removed;
        out = 0;
    }
    if (was_live && !out) ++t.died;
    if (!was_live && out) ++t.born;
    return out;
}

// Adds a 128-bit value into four 64-bit limb counters (no return values).
__device__ __forceinline__ void red_add_limbs(unsigned long long* c, const U128& x) {
    const unsigned long long l[4] = {x.lo & 0xffffffffull, x.lo >> 32, x.hi & 0xffffffffull,
                                     x.hi >> 32};
#pragma unroll
    for (int q = 0; q < 4; ++q)
        if (l[q]) atomicAdd(c + q, l[q]);
}
// The limb counters' exact 128-bit total.
__device__ __forceinline__ U128 limbs_total(const unsigned long long (&c)[4]) {
    U128 t{c[0], 0ull};
    u128_add(t, U128{c[1] << 32, c[1] >> 32});
    u128_add(t, U128{0ull, c[2]});
    u128_add(t, U128{0ull, c[3] << 32});
    return t;
}

// Block totals of a pass, then one set of reductions into rotation r's stat slot.
// Warp total of a 128-bit sum: sixteen-bit limbs summed by warp reductions
// (each limb total stays below 2^21) and recombined exactly.
__device__ __forceinline__ U128 warp_sum_u128(const U128& x) {
    U128 t{0ull, 0ull};
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const unsigned long long word = q < 4 ? x.lo : x.hi;
        const unsigned limb = (unsigned)(word >> (16 * (q & 3))) & 0xffffu;
        const unsigned long long sum = __reduce_add_sync(0xffffffffu, limb);
        const int sh = 16 * q;
        U128 part;
        if (sh < 64) {
            part.lo = sum << sh;
            part.hi = sh ? (sum >> (64 - sh)) : 0ull;
        } else {
            part.lo = 0ull;
            part.hi = sum << (sh - 64);
        }
        u128_add(t, part);
    }
    return t;
}

// Warp total of a tally (every lane holds it; all lanes must call).
__device__ __forceinline__ void warp_tally(PairTally& t) {
    t.born = __reduce_add_sync(0xffffffffu, t.born);
    t.died = __reduce_add_sync(0xffffffffu, t.died);
    t.flags = __reduce_or_sync(0xffffffffu, t.flags);
    t.radii = __reduce_add_sync(0xffffffffu, t.radii);
    if (__any_sync(0xffffffffu, t.removed != 0u)) {
        t.removed = __reduce_add_sync(0xffffffffu, t.removed);
        t.l1 = warp_sum_u128(t.l1);
        t.sq = warp_sum_u128(t.sq);
    }
}

template <int NT>
__device__ __forceinline__ void flush_tally(const HashArgs& a, unsigned r, PairTally t,
                                            PairTally* s_t) {
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    warp_tally(t);
    if (lane == 0) s_t[warp] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long born = 0, died = 0, removed = 0, radii = 0;
        unsigned flags = 0;
        U128 l1{0ull, 0ull}, sq{0ull, 0ull};
        for (int w = 0; w < NT / 32; ++w) {
            born += s_t[w].born;
            died += s_t[w].died;
            removed += s_t[w].removed;
            radii += s_t[w].radii;
            flags |= s_t[w].flags;
            u128_add(l1, s_t[w].l1);
            u128_add(sq, s_t[w].sq);
        }
        HashStat* hs = a.stats + (size_t)r * kStatSlots + (blockIdx.x % kStatSlots);
        red_add_limbs(hs->l1, l1);
        red_add_limbs(hs->sq, sq);
        if (born) atomicAdd(&hs->born, born);
        if (died) atomicAdd(&hs->died, died);
        if (removed) atomicAdd(&hs->removed, removed);
        if (radii) atomicAdd(&hs->radii, radii);
        if (flags) atomicOr(&hs->flags, flags);
    }
}

// Validated rotation: the merged radii of a pair's two output keys
// (tpgp_rev.c:459-464 per child, :699-706 per merge).  Each live member
// sends a cos child to itself with radius upadd(upmul(|v|, rc),
// round_radius(v c)) and a sin child to its partner with radius
// upadd(upmul(|v|, rs), round_radius(v s)); a key's radius is the upadd of
// its contributions' radii and, where two nonzero contributions meet, the
// rounding radius of their sum.  Nonzero merged radii are logged (tagged);
// a nonfinite child or merged radius is ENUMERIC.
template <int W>
__device__ __forceinline__ void pair_radii(const HashArgs& a, const PassParams& p, const Key<W>& K,
                                           const Key<W>& P, bool k_live, bool p_live, double vk,
                                           double vp, double nk, double np, PairTally& t) {
    double kc = 0.0, ks = 0.0, pc = 0.0, ps = 0.0;  // child radii: K's cos / sin, P's cos / sin
    double xk = 0.0, yk = 0.0, xp = 0.0, yp = 0.0;  // the children's values (before signs)
    if (k_live) {
        xk = __dmul_rn(vk, p.c);
        yk = __dmul_rn(vk, p.s);
        kc = up_add(up_mul(abs_of(vk), p.rc), rounding_radius(xk));
        ks = up_add(up_mul(abs_of(vk), p.rs), rounding_radius(yk));
    }
    if (p_live) {
        xp = __dmul_rn(vp, p.c);
        yp = __dmul_rn(vp, p.s);
        pc = up_add(up_mul(abs_of(vp), p.rc), rounding_radius(xp));
        ps = up_add(up_mul(abs_of(vp), p.rs), rounding_radius(yp));
    }
    double rk, rp;
    if (k_live && p_live) {
        rk = up_add(kc, ps);
        if (!is_zero(xk) && !is_zero(yp)) rk = up_add(rk, rounding_radius(nk));
        rp = up_add(pc, ks);
        if (!is_zero(xp) && !is_zero(yk)) rp = up_add(rp, rounding_radius(np));
    } else if (k_live) {
        rk = kc;
        rp = ks;
    } else {
        rk = ps;
        rp = pc;
    }
    if (!is_finite(kc) || !is_finite(ks) || !is_finite(pc) || !is_finite(ps) || !is_finite(rk) ||
        !is_finite(rp))
        t.flags |= ST_NUMERIC;
    if (!is_zero(rk)) {
        log_entry<W>(a, K, dbits(rk) | kSignBit);
        ++t.radii;
    }
    if (!is_zero(rp)) {
        log_entry<W>(a, P, dbits(rp) | kSignBit);
        ++t.radii;
    }
}

// Index 4 pi + pj of a key's two site symbols in the pass's branch tables.
template <int W>
__device__ __forceinline__ unsigned pass_index(const PassParams& p, const Key<W>& k) {
    const unsigned pi = site_symbol(word_at<W>(k, p.i_word), p.i_shift);
    const unsigned pj = site_symbol(word_at<W>(k, p.j_word), p.j_shift);
    return 4u * pi + pj;
}

// One rotation over the occupied slots, in rounds of NT list entries per
// CTA.  Phase 1: every thread reads one list entry (key, slot, stamp) and
// classifies the key; a commuting key needs no work once every value has
// passed the threshold (else its value is re-thresholded in place), and an
// anticommuting key (typically a small fraction) is queued in shared memory.
// Phase 2: the queued keys, packed into the first warps, each load their
// slot's record and the partner's first probe record at once, and the
// pair's owner updates it.  Entries appended during the pass (this pass's
// stamp, or not yet written) are skipped.  Inserts reserve their list
// entries with one warp atomic issued together with their slot claims.
//
// The first round's entries are loaded without waiting for the list length:
// entries past the length are unwritten (the list starts filled with all
// ones), and entries appended by this pass carry this pass's stamp.
// V: validated rotations (error radii), a separate instantiation so the
// plain pass keeps its registers.
template <int W, int NT, bool V = false>
__device__ __forceinline__ void hash_pass(const HashArgs& a, const PassParams& p, unsigned r,
                                          unsigned k) {
    __shared__ PairTally s_t[NT / 32];
    __shared__ Key<W> s_key[NT];
    __shared__ uint32_t s_slot[NT];
    __shared__ unsigned char s_idx[NT];
    __shared__ unsigned s_n;
    __shared__ unsigned long long s_len;
    const uint32_t stamp = k + 2u;  // pass k: stamps; rotation r: parameters
    Key<W> Q;
#pragma unroll
    for (int w = 0; w < W; ++w) Q.w[w] = p.mask[w];
    const double c = p.c, s = p.s;
    PairTally t = empty_tally();
    const unsigned long long S = a.slots;  // also the list's capacity
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const unsigned long long stride = (unsigned long long)gridDim.x * NT;
    unsigned long long base = (unsigned long long)blockIdx.x * NT;
    Entry<W> E;
    E.slot = kNoSlot;
    E.stamp = 0u;
    if (base + threadIdx.x < S) E = load_entry<W>(a.occ, base + threadIdx.x);
    if (threadIdx.x == 0) {
        s_len = min(__ldcg(a.claimed), S);
        s_n = 0u;
    }
    for (;;) {
        // ---- phase 1: classify, queue the anticommuting keys
        bool anti = false;
        unsigned idx = 0;
        if (E.slot != kNoSlot && E.stamp < stamp) {
            idx = pass_index<W>(p, E.key);
            anti = (p.anti >> idx) & 1u;
            if (!anti && !p.settled) {
                // commuting: merged value v + 0 = v, still subject to the
                // threshold like every merged term (no anticommuting key pairs with it)
                const unsigned long long v = load_rec<W>(a.rec, E.slot).val;
                if (v) {
                    const unsigned long long out = settle<W>(p, E.key, from_bits(v), true, t);
                    if (out != v) store_val<W>(a.rec, E.slot, out);
                    if (a.xlog_keys && !out && !is_zero(from_bits(v)))
                        log_removed<W>(a, E.key, from_bits(v));
                }
            }
        }
        __syncthreads();  // s_n = 0 and s_len visible; the previous round's queue consumed
        const unsigned m = __ballot_sync(0xffffffffu, anti);
        if (m) {
            const unsigned leader = (unsigned)(__ffs(m) - 1);
            unsigned at = 0;
            if (lane == leader) at = atomicAdd(&s_n, (unsigned)__popc(m));
            at = __shfl_sync(0xffffffffu, at, leader) + __popc(m & lanemask_lt());
            if (anti) {
                s_key[at] = E.key;
                s_slot[at] = E.slot;
                s_idx[at] = (unsigned char)idx;
            }
        }
        __syncthreads();
        const unsigned n = s_n;
        const unsigned long long len = s_len;
        // ---- phase 2: the queued keys, one per thread of the first warps
        if (warp * 32u < n) {
            const unsigned q = warp * 32u + lane;
            bool want = false;  // this lane inserts its partner P with value pbits at empty_at
            Key<W> P;
            unsigned long long pbits = 0, empty_at = 0;
            if (q < n) {
                const Key<W> K = s_key[q];
                const unsigned long long slot = s_slot[q];
                const unsigned qidx = s_idx[q];
                P = key_xor<W>(K, Q);
                const unsigned long long ps = slot_of(hash_of<W>(P), S);
                const Rec<W> R = load_rec<W>(a.rec, slot);
                unsigned long long pb = 0;
                bool overflow = false;
                const long long found =
                    probe_from<W>(a, P, ps, load_rec<W>(a.rec, ps), stamp, &empty_at, &pb, &overflow);
                if (overflow) {
                    t.flags |= ST_TABLE;
                } else if ((found < 0 || key_less<W>(K, P)) && (R.val | pb)) {
                    // this thread owns the pair, and at least one member is live
                    const bool k_live = R.val != 0ull, p_live = pb != 0ull;
                    const bool plus_k = (p.plus >> qidx) & 1u;
                    const bool plus_p = (p.plus >> (qidx ^ p.qmix)) & 1u;
                    double nk, np;
                    if (k_live) {
                        const double v = from_bits(R.val);
                        double sk = __dmul_rn(v, s);  // K's sin child, landing on P
                        if (!plus_k) sk = negate(sk);
                        nk = __dmul_rn(v, c);
                        np = sk;
                        if (p_live) {
                            const double vp = from_bits(pb);
                            double sp = __dmul_rn(vp, s);  // P's sin child, landing on K
                            if (!plus_p) sp = negate(sp);
                            nk = __dadd_rn(nk, sp);
                            np = __dadd_rn(__dmul_rn(vp, c), sk);
                        }
                    } else {
                        const double vp = from_bits(pb);
                        double sp = __dmul_rn(vp, s);
                        if (!plus_p) sp = negate(sp);
                        nk = sp;
                        np = __dmul_rn(vp, c);
                    }
                    const unsigned long long kbits = settle<W>(p, K, nk, k_live, t);
                    pbits = settle<W>(p, P, np, p_live, t);
                    if constexpr (V)
                        pair_radii<W>(a, p, K, P, k_live, p_live, from_bits(R.val), from_bits(pb), nk, np, t);
                    if (a.xlog_keys) {
                        if (!kbits && !is_zero(nk)) log_removed<W>(a, K, nk);
                        if (!pbits && !is_zero(np)) log_removed<W>(a, P, np);
                    }
                    if (kbits != R.val) store_val<W>(a.rec, slot, kbits);
                    if (found >= 0) {
                        if (pbits != pb) store_val<W>(a.rec, (unsigned long long)found, pbits);
                    } else {
                        want = pbits != 0ull;
                    }
                }
            }
            // inserts: the warp's list reservation and the lanes' slot claims in flight together
            const unsigned mi = __ballot_sync(0xffffffffu, want);
            if (mi) {
                const unsigned leader = (unsigned)(__ffs(mi) - 1);
                unsigned long long at = 0;
                uint32_t old = 1u;
                if (lane == leader) at = atomicAdd(a.claimed, (unsigned long long)__popc(mi));
                if (want) old = atomicCAS(rec_tag<W>(a.rec, empty_at), 0u, stamp);
                at = __shfl_sync(0xffffffffu, at, leader) + __popc(mi & lanemask_lt());
                if (want) {
                    long long ns = -1;
                    if (old == 0u) {
                        unsigned long long* d = a.rec + empty_at * rec_words<W>();
#pragma unroll
                        for (int w = 0; w < W; ++w) d[w] = P.w[w];
                        d[W] = pbits;
                        ns = (long long)empty_at;
                    } else {  // another insert took the slot: the next empty one
                        bool ovf = false;
                        ns = hash_insert<W>(a, P, pbits, next_slot(empty_at, S), stamp, &ovf);
                    }
                    if (ns >= 0 && at < S) store_entry<W>(a.occ, at, P, (unsigned long long)ns, stamp);
                    else t.flags |= ST_TABLE;
                }
            }
        }
        base += stride;  // block-uniform
        if (base >= len) break;
        E.slot = kNoSlot;
        if (base + threadIdx.x < len) E = load_entry<W>(a.occ, base + threadIdx.x);
        __syncthreads();  // every thread has read s_n before it is cleared
        if (threadIdx.x == 0) s_n = 0u;
    }
    flush_tally<NT>(a, r, t, s_t);
}

// Launched with programmatic stream serialization (hash_pdl), a pass's CTAs
// become resident while the previous pass drains and wait here for its
// completion and memory; launched plainly, pdl_enter returns at once.
template <int W, bool V = false>
__global__ void __launch_bounds__(kHashBlock, 4) k_hash_rotate(HashArgs a, PassParams p, unsigned r,
                                                               unsigned k) {
    pdl_enter();
    hash_pass<W, kHashBlock, V>(a, p, r, k);
}

// All rotations of a step in one cooperative launch (one CTA of 1024 threads
// per SM), a bounded grid barrier between rotations; a barrier that gives up
// sets ST_TIMEOUT and the CTA leaves.  The passes are those of k_hash_rotate.
constexpr int kHashPersistentBlock = 1024;
template <int W>
__global__ void __launch_bounds__(kHashPersistentBlock, 1) k_hash_rotate_all(HashArgs a) {
    for (unsigned r = 0; r < a.rotations; ++r) {
        hash_pass<W, kHashPersistentBlock>(a, pass_params(a.ps[r]), r, r);
        if (!grid_barrier(a.st)) return;
    }
}

// ------------------------------------------------- fused runs on one site pair
// A run of consecutive rotations on the same two sites (a secular edge's ZZ,
// XX, YY; six at the middle of a Strang step) whose generators span a group
// G of at most four XOR patterns G = {0, b1, b2, b1 ^ b2}.  Every key's coset
// K xor G is closed under each rotation of the run, so each coset is evolved
// on its own through the whole run -- per rotation exactly the pair rule of
// hash_pass (commuting members keep v + 0, anticommuting members combine
// with their partner a ^ label(Q)), with the zero drop, threshold and
// removed-weight sums of that rotation -- and only the final values are
// written.  The coset is owned by its smallest member present when the pass
// starts; results are those of the run's rotations one by one.
constexpr int kMaxRun = 6;

template <int W>
__device__ __forceinline__ void coset_sign(const RotParams& p, const Key<W>& m, bool& anti,
                                           bool& plus) {
    branch_info(p, word_at<W>(m, p.i_word), word_at<W>(m, p.j_word), anti, plus);
}

// Whether a key anticommutes with some generator of the run.  A key that
// commutes with all of them keeps its value through the run (no flipped
// child lands on a commuting key), so only the threshold can change it;
// and a member of a coset that does anticommute has every pairing partner
// anticommuting too, so the run's pairings stay among such members.
template <int W>
__device__ __forceinline__ bool run_participates(const HashArgs& a, unsigned r0, unsigned L,
                                                 const Key<W>& key) {
    for (unsigned l = 0; l < L; ++l) {
        bool anti, plus;
        coset_sign<W>(a.ps[r0 + l], key, anti, plus);
        if (anti) return true;
    }
    return false;
}

template <int W>
__global__ void __launch_bounds__(kHashBlock, 2) k_hash_run(HashArgs a, unsigned k) {
    __shared__ unsigned long long s_acc[kMaxRun][4];
    __shared__ unsigned s_cnt[kMaxRun][3];  // born, died, removed
    __shared__ unsigned s_flags;
    for (int q = threadIdx.x; q < kMaxRun * 4; q += blockDim.x) (&s_acc[0][0])[q] = 0ull;
    for (int q = threadIdx.x; q < kMaxRun * 3; q += blockDim.x) (&s_cnt[0][0])[q] = 0u;
    if (threadIdx.x == 0) s_flags = 0u;
    __syncthreads();
    const uint2 run = a.runs[k];
    const unsigned r0 = run.x, L = run.y;
    const uint32_t stamp = k + 2u;
    // the run's group: G[1] = the first mask, G[2] the first other mask
    Key<W> G[4];
#pragma unroll
    for (int w = 0; w < W; ++w) G[0].w[w] = 0ull;
    G[1] = mask_key<W>(a.ps[r0]);
    G[2] = G[0];
    bool has_b2 = false;
    for (unsigned l = 1; l < L; ++l) {
        const Key<W> q = mask_key<W>(a.ps[r0 + l]);
        if (!has_b2 && !key_eq<W>(q, G[1])) {
            G[2] = q;
            has_b2 = true;
        }
    }
    G[3] = key_xor<W>(G[1], G[2]);
    const int gs = has_b2 ? 4 : 2;
    // after the step's first pass every value has passed the threshold once
    const bool settled = k > 0 && a.ps[r0 - 1].threshold_bits == a.ps[r0].threshold_bits;
    unsigned flags = 0u;
    const unsigned long long S = a.slots;
    const unsigned long long len = min(__ldcg(a.claimed), S);
    const unsigned lane = threadIdx.x & 31u;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u);
         base < len; base += stride) {
        const unsigned long long i = base + lane;
        // a coset inserts at most three members: appended after the work
        bool ins[4] = {false, false, false, false};
        unsigned long long ins_slot[4] = {0, 0, 0, 0};
        Key<W> ins_key[4];
        Entry<W> E;
        E.slot = kNoSlot;
        E.stamp = stamp;
        if (i < len) E = load_entry<W>(a.occ, i);
        const uint32_t slot = E.slot;
        Rec<W> R;
        R.tag = stamp;
        bool part = false;
        if (slot != kNoSlot && E.stamp < stamp) {
            part = run_participates<W>(a, r0, L, E.key);
            if (part || !settled) R = load_rec<W>(a.rec, slot);
        }
        if (R.tag < stamp && !part) {
            // commutes with the whole run: the run's first rotation thresholds
            // the unchanged value, the later ones see the same value
            if (R.val) {
                PairTally t = empty_tally();
                const unsigned long long out = settle<W>(a.ps[r0], R.key, from_bits(R.val), true, t);
                if (out != R.val) store_val<W>(a.rec, slot, out);
                if (t.removed) {
                    shared_add_u128(s_acc[0], t.l1);
                    shared_add_u128(s_acc[0] + 2, t.sq);
                    atomicAdd(&s_cnt[0][2], t.removed);
                }
                if (t.died) atomicAdd(&s_cnt[0][1], t.died);
                flags |= t.flags;
            }
        } else if (R.tag < stamp) {
            // the coset's other members: first probe records loaded together
            // (only those that take part in the run; the others keep to themselves)
            Key<W> M[4];
            Rec<W> PR[4];
            unsigned long long ps[4], ea[4], v[4];
            long long sl[4];
            M[0] = R.key;
            sl[0] = (long long)slot;
            v[0] = R.val;
            ea[0] = 0ull;
            bool mp[4];
            mp[0] = true;
#pragma unroll
            for (int m = 1; m < 4; ++m) {
                M[m] = key_xor<W>(R.key, G[m]);
                sl[m] = -1;
                v[m] = 0ull;
                ea[m] = 0ull;
                mp[m] = m < gs && run_participates<W>(a, r0, L, M[m]);
                if (mp[m]) {
                    ps[m] = slot_of(hash_of<W>(M[m]), S);
                    PR[m] = load_rec<W>(a.rec, ps[m]);
                }
            }
            bool overflow = false;
#pragma unroll
            for (int m = 1; m < 4; ++m) {
                if (!mp[m]) continue;  // absent from the run's pairings: never probed, never written
                sl[m] = probe_from<W>(a, M[m], ps[m], PR[m], stamp, &ea[m], &v[m], &overflow);
            }
            // owner: the smallest present member; a coset with no live member has nothing to do
            bool own = !overflow;
            unsigned long long any = v[0];
#pragma unroll
            for (int m = 1; m < 4; ++m) {
                if (m >= gs) continue;
                any |= v[m];
                if (sl[m] >= 0 && key_less<W>(M[m], M[0])) own = false;
            }
            if (overflow) flags |= ST_TABLE;
            if (own && any) {
                double x[4];
                bool live[4];
#pragma unroll
                for (int m = 0; m < 4; ++m) {
                    live[m] = v[m] != 0ull;
                    x[m] = from_bits(v[m]);
                }
                for (unsigned l = 0; l < L; ++l) {
                    const RotParams& p = a.ps[r0 + l];
                    const Key<W> q = mask_key<W>(p);
                    const int b = key_eq<W>(q, G[1]) ? 1 : (key_eq<W>(q, G[2]) ? 2 : 3);
                    const double c = p.c, s = p.s;
                    bool anti[4], plus[4];
#pragma unroll
                    for (int m = 0; m < 4; ++m) coset_sign<W>(p, M[m], anti[m], plus[m]);
                    double nx[4];
                    bool touched[4];
#pragma unroll
                    for (int m = 0; m < 4; ++m) {
                        nx[m] = 0.0;
                        touched[m] = false;
                        if (m >= gs) continue;
                        if (!anti[m]) {
                            nx[m] = x[m];
                            touched[m] = live[m];
                            continue;
                        }
                        const int pb = m ^ b;
                        const bool lp = pick<4, bool>(live, pb);
                        double sp = __dmul_rn(pick<4, double>(x, pb), s);  // partner's sin child
                        if (!pick<4, bool>(plus, pb)) sp = negate(sp);
                        if (live[m] && lp) nx[m] = __dadd_rn(__dmul_rn(x[m], c), sp);
                        else if (live[m]) nx[m] = __dmul_rn(x[m], c);
                        else if (lp) nx[m] = sp;
                        touched[m] = live[m] || lp;
                    }
                    PairTally t = empty_tally();
#pragma unroll
                    for (int m = 0; m < 4; ++m) {
                        if (!touched[m]) continue;  // absent before and after: no term
                        const unsigned long long out = settle<W>(p, M[m], nx[m], live[m], t);
                        live[m] = out != 0ull;
                        x[m] = from_bits(out);
                    }
                    if (t.removed) {
                        shared_add_u128(s_acc[l], t.l1);
                        shared_add_u128(s_acc[l] + 2, t.sq);
                    }
                    if (t.born) atomicAdd(&s_cnt[l][0], t.born);
                    if (t.died) atomicAdd(&s_cnt[l][1], t.died);
                    if (t.removed) atomicAdd(&s_cnt[l][2], t.removed);
                    flags |= t.flags;
                }
#pragma unroll
                for (int m = 0; m < 4; ++m) {
                    if (m >= gs) continue;
                    const unsigned long long bits = live[m] ? dbits(x[m]) : 0ull;
                    if (sl[m] >= 0) {
                        if (bits != v[m]) store_val<W>(a.rec, (unsigned long long)sl[m], bits);
                    } else if (bits) {
                        bool ovf = false;
                        const long long ns = hash_insert<W>(a, M[m], bits, ea[m], stamp, &ovf);
                        if (ns >= 0) {
                            ins[m] = true;
                            ins_slot[m] = (unsigned long long)ns;
                            ins_key[m] = M[m];
                        } else {
                            flags |= ST_TABLE;
                        }
                    }
                }
            }
        }
#pragma unroll
        for (int m = 1; m < 4; ++m) {
            const unsigned long long at = list_reserve(a, ins[m]);
            if (ins[m]) {
                if (at < S) store_entry<W>(a.occ, at, ins_key[m], ins_slot[m], stamp);
                else flags |= ST_TABLE;
            }
        }
    }
    if (flags) atomicOr(&s_flags, flags);
    __syncthreads();
    if (threadIdx.x == 0) {
        for (unsigned l = 0; l < L; ++l) {
            HashStat* hs = a.stats + (size_t)(r0 + l) * kStatSlots + (blockIdx.x % kStatSlots);
            red_add_limbs(hs->l1, U128{s_acc[l][0], s_acc[l][1]});
            red_add_limbs(hs->sq, U128{s_acc[l][2], s_acc[l][3]});
            if (s_cnt[l][0]) atomicAdd(&hs->born, (unsigned long long)s_cnt[l][0]);
            if (s_cnt[l][1]) atomicAdd(&hs->died, (unsigned long long)s_cnt[l][1]);
            if (s_cnt[l][2]) atomicAdd(&hs->removed, (unsigned long long)s_cnt[l][2]);
            if (s_flags) atomicOr(&hs->flags, s_flags);
        }
    }
}

// --------------------------------------------------------------- commit chain
// Per-rotation totals, one warp per rotation: the 32 stat slots summed
// exactly, the fixed-point sums converted up (l1, sq) and l2 = nextUp(sqrt(sq)),
// as commit_rotation computes them.
struct HashRot {
    double l1, sq, l2;
    long long dn;                  // born - died
    unsigned long long removed;
    unsigned flags, pad;           // pad: the exact ledger's sort notes its result half here
    unsigned long long radii;      // merged radii logged (validated rotations)
    double ar;                     // upper L2 of the merged radii (validated rotations)
};

__global__ void __launch_bounds__(256) k_hash_reduce(HashArgs a, HashRot* rot) {
    const unsigned r = blockIdx.x * 8u + (threadIdx.x >> 5), lane = threadIdx.x & 31u;
    if (r >= a.rotations) return;
    const HashStat& x = a.stats[(size_t)r * kStatSlots + lane];
    U128 l1 = limbs_total(x.l1), sq = limbs_total(x.sq);
    unsigned long long born = x.born, died = x.died, removed = x.removed, radii = x.radii;
    unsigned flags = x.flags;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        u128_add(l1, shfl_down_u128(l1, off));
        u128_add(sq, shfl_down_u128(sq, off));
        born += __shfl_down_sync(0xffffffffu, born, off);
        died += __shfl_down_sync(0xffffffffu, died, off);
        removed += __shfl_down_sync(0xffffffffu, removed, off);
        radii += __shfl_down_sync(0xffffffffu, radii, off);
        flags |= __shfl_down_sync(0xffffffffu, flags, off);
    }
    if (lane == 0) {
        const RotParams& p = a.ps[r];
        HashRot h;
        h.l1 = u128_to_double_up(l1, p.fx_unit1);
        h.sq = u128_to_double_up(sq, p.fx_unit2);
        h.l2 = h.sq == 0.0 ? 0.0 : next_up(sqrt(h.sq));
        h.dn = (long long)(born - died);
        h.removed = removed;
        h.flags = flags;
        h.pad = 0;
        h.radii = radii;
        h.ar = 0.0;
        rot[r] = h;
    }
}

// ---------------------------------------------------------------- exact ledger
// The reference adds each rotation's removed |v| in key order as its merge
// loop meets them (tpgp_rev.c:716-729; upper_l2 :43-63 without MPFR).  The
// passes log them per rotation in any order, so after the passes:
//   k_hash_xstarts: segment starts = exclusive scan of the removed counts;
//   k_hash_xsort:   each segment sorted by key by one CTA (keys are unique
//                   within a rotation: a key is in one pair per rotation);
//   k_hash_xchains: one warp per rotation adds its segment sequentially.

// One CTA of 1024 threads: starts[r] for r <= R; ST_LOG when the log
// overflowed, ST_ORDER when the counts and the log disagree.  Clears the
// sort's segment counter.
__global__ void __launch_bounds__(1024) k_hash_xstarts(HashArgs a, const HashRot* rot,
                                                       unsigned long long* starts,
                                                       unsigned* next_segment) {
    __shared__ unsigned long long s_part[32];
    __shared__ unsigned long long s_carry;
    const unsigned R = a.rotations, tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) {
        s_carry = 0ull;
        *next_segment = 0u;
    }
    __syncthreads();
    for (unsigned base = 0; base < R; base += 1024) {
        const unsigned r = base + tid;
        const unsigned long long mine = r < R ? rot[r].removed + rot[r].radii : 0ull;
        unsigned long long incl = mine;  // warp inclusive scan
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= (unsigned)off) incl += y;
        }
        if (lane == 31) s_part[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            unsigned long long w = s_part[lane], wi = w;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const unsigned long long y = __shfl_up_sync(0xffffffffu, wi, off);
                if (lane >= (unsigned)off) wi += y;
            }
            s_part[lane] = wi - w;  // exclusive warp offsets
        }
        __syncthreads();
        if (r < R) starts[r] = s_carry + s_part[warp] + incl - mine;
        __syncthreads();
        if (tid == 1023) s_carry += s_part[31] + incl;  // chunk total (thread 1023 ends it)
        __syncthreads();
    }
    if (tid == 0) {
        starts[R] = s_carry;
        const unsigned long long total = *a.xlog_count;
        if (total > a.xlog_cap) atomicOr(&a.st->status, ST_LOG);
        else if (total != s_carry) atomicOr(&a.st->status, ST_ORDER);
    }
}

// Segment sort: a stable LSD radix sort by key of each rotation's segment,
// one CTA per segment (taken from a counter), on the onesweep tile scheme
// without look-back (the CTA owns every tile of its segment, in order):
// the histograms of all digits in one pass over the segment, then one
// scatter pass per digit that is not constant over the segment, tile by
// tile through shared memory, between the log's two halves.  A segment of
// one tile stays in registers and shared memory for all its passes.  The
// half that holds the sorted segment is noted in the rotation's HashRot.pad.
template <int W>
__host__ __device__ constexpr size_t xsort_smem() {
    return (size_t)kOsTile * (8 * W + 8) + (size_t)8 * W * 256 * 4;
}

template <int W>
__global__ void __launch_bounds__(kOsBlock) k_hash_xsort(HashArgs a, const unsigned long long* starts,
                                                         unsigned* next_segment, uint64_t* k1,
                                                         unsigned long long* v1, HashRot* rot,
                                                         int digits) {
    extern __shared__ __align__(16) unsigned char xs_raw[];
    uint64_t* st_k = reinterpret_cast<uint64_t*>(xs_raw);  // [tile][W]
    unsigned long long* st_v = reinterpret_cast<unsigned long long*>(st_k + (size_t)kOsTile * W);
    unsigned* s_h = reinterpret_cast<unsigned*>(st_v + kOsTile);  // [digit][256]: counts, then bases
    __shared__ unsigned s_cnt[256], s_local[256], s_runt[256], s_run[256];
    __shared__ unsigned s_w[kOsBlock / 32][256];
    __shared__ unsigned s_part[kOsBlock / 32];
    __shared__ unsigned s_seg, s_const;
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    uint64_t* const k0 = a.xlog_keys;
    unsigned long long* const v0 = a.xlog_vals;
    const int D = digits;
    for (;;) {
        __syncthreads();
        if (tid == 0)
            s_seg = *reinterpret_cast<volatile unsigned*>(&a.st->status) ? a.rotations
                                                                          : atomicAdd(next_segment, 1u);
        __syncthreads();
        const unsigned r = s_seg;
        if (r >= a.rotations) return;
        const unsigned long long b = starts[r];
        const unsigned n = (unsigned)(starts[r + 1] - b);
        if (n <= 1) {
            if (tid == 0) rot[r].pad = 0u;  // in the log's first half already
            continue;
        }
        // histograms of every digit over the segment
        for (int q = tid; q < D * 256; q += kOsBlock) s_h[q] = 0u;
        __syncthreads();
        for (unsigned i = tid; i < n; i += kOsBlock) {
            const Key<W> k = load_key<W>(k0, b + i);
            for (int d = 0; d < D; ++d) atomicAdd(&s_h[d * 256 + sort_digit<W>(k, d)], 1u);
        }
        __syncthreads();
        // exclusive bases per digit; a digit whose one bucket holds the whole
        // segment is constant (its pass would not move anything): mark its
        // bucket count as ~0u
        for (int d = 0; d < D; ++d) {
            const unsigned c = s_h[d * 256 + tid];
            if (tid == 0) s_const = 0u;
            __syncthreads();
            if (c == n) s_const = 1u;
            unsigned incl = c;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const unsigned y = __shfl_up_sync(0xffffffffu, incl, off);
                if (lane >= (unsigned)off) incl += y;
            }
            if (lane == 31) s_part[warp] = incl;
            __syncthreads();
            unsigned before = 0;
            for (unsigned w = 0; w < warp; ++w) before += s_part[w];
            const bool skip = s_const != 0u;
            __syncthreads();
            s_h[d * 256 + tid] = skip ? ~0u : before + incl - c;
        }
        __syncthreads();
        int half = 0;  // which half holds the segment's current order
        if (n <= (unsigned)kOsTile) {
            // one tile: registers and shared memory only
            Key<W> key[kOsItems];
            unsigned long long val[kOsItems];
#pragma unroll
            for (int e = 0; e < kOsItems; ++e) {
                const unsigned i = (unsigned)e * kOsBlock + tid;
                if (i < n) {
                    key[e] = load_key<W>(k0, b + i);
                    val[e] = __ldcg(v0 + b + i);
                }
            }
            for (int d = 0; d < D; ++d) {
                if (s_h[d * 256] == ~0u) continue;  // constant digit (uniform read)
                unsigned dig[kOsItems];
                s_cnt[tid] = 0u;
                s_runt[tid] = 0u;
                __syncthreads();
#pragma unroll
                for (int e = 0; e < kOsItems; ++e) {
                    const unsigned i = (unsigned)e * kOsBlock + tid;
                    dig[e] = i < n ? sort_digit<W>(key[e], d) : 256u;
                }
                // the tile's bucket offsets are the segment's bases
#pragma unroll
                for (int e = 0; e < kOsItems; ++e) {
                    for (int q = lane; q < 256; q += 32) s_w[warp][q] = 0u;
                    __syncthreads();
                    const unsigned peers = __match_any_sync(0xffffffffu, dig[e]);
                    if (dig[e] < 256u && lane == (unsigned)(__ffs(peers) - 1)) s_w[warp][dig[e]] = __popc(peers);
                    __syncthreads();
                    if (dig[e] < 256u) {
                        unsigned bw = 0;
                        for (unsigned w = 0; w < warp; ++w) bw += s_w[w][dig[e]];
                        const unsigned pos = s_h[d * 256 + dig[e]] + s_runt[dig[e]] + bw +
                                             __popc(peers & lanemask_lt());
#pragma unroll
                        for (int w = 0; w < W; ++w) st_k[(size_t)pos * W + w] = key[e].w[w];
                        st_v[pos] = val[e];
                    }
                    __syncthreads();
                    unsigned tot = 0;
#pragma unroll
                    for (int w = 0; w < kOsBlock / 32; ++w) tot += s_w[w][tid];
                    s_runt[tid] += tot;
                    __syncthreads();
                }
#pragma unroll
                for (int e = 0; e < kOsItems; ++e) {
                    const unsigned i = (unsigned)e * kOsBlock + tid;
                    if (i < n) {
#pragma unroll
                        for (int w = 0; w < W; ++w) key[e].w[w] = st_k[(size_t)i * W + w];
                        val[e] = st_v[i];
                    }
                }
                __syncthreads();
            }
#pragma unroll
            for (int e = 0; e < kOsItems; ++e) {
                const unsigned i = (unsigned)e * kOsBlock + tid;
                if (i < n) {
                    store_key<W>(k1, b + i, key[e]);
                    v1[b + i] = val[e];
                }
            }
            if (tid == 0) rot[r].pad = 1u;
            continue;
        }
        for (int d = 0; d < D; ++d) {
            if (s_h[d * 256] == ~0u) continue;  // constant digit
            const uint64_t* sk = half ? k1 : k0;
            const unsigned long long* sv = half ? v1 : v0;
            uint64_t* dk = half ? k0 : k1;
            unsigned long long* dv = half ? v0 : v1;
            s_run[tid] = s_h[d * 256 + tid];  // where the bucket's next item goes
            for (unsigned t0 = 0; t0 < n; t0 += kOsTile) {
                __syncthreads();
                s_cnt[tid] = 0u;
                s_runt[tid] = 0u;
                __syncthreads();
                Key<W> key[kOsItems];
                unsigned long long val[kOsItems];
                unsigned dig[kOsItems];
#pragma unroll
                for (int e = 0; e < kOsItems; ++e) {
                    const unsigned i = t0 + (unsigned)e * kOsBlock + tid;
                    dig[e] = 256u;
                    if (i < n) {
                        key[e] = load_key<W>(sk, b + i);
                        val[e] = __ldcg(sv + b + i);
                        dig[e] = sort_digit<W>(key[e], d);
                        atomicAdd(&s_cnt[dig[e]], 1u);
                    }
                }
                __syncthreads();
                {  // exclusive scan of the tile's counts
                    const unsigned c = s_cnt[tid];
                    unsigned incl = c;
#pragma unroll
                    for (int off = 1; off < 32; off <<= 1) {
                        const unsigned y = __shfl_up_sync(0xffffffffu, incl, off);
                        if (lane >= (unsigned)off) incl += y;
                    }
                    if (lane == 31) s_part[warp] = incl;
                    __syncthreads();
                    unsigned before = 0;
                    for (unsigned w = 0; w < warp; ++w) before += s_part[w];
                    s_local[tid] = before + incl - c;
                }
#pragma unroll
                for (int e = 0; e < kOsItems; ++e) {
                    for (int q = lane; q < 256; q += 32) s_w[warp][q] = 0u;
                    __syncthreads();
                    const unsigned peers = __match_any_sync(0xffffffffu, dig[e]);
                    if (dig[e] < 256u && lane == (unsigned)(__ffs(peers) - 1)) s_w[warp][dig[e]] = __popc(peers);
                    __syncthreads();
                    if (dig[e] < 256u) {
                        unsigned bw = 0;
                        for (unsigned w = 0; w < warp; ++w) bw += s_w[w][dig[e]];
                        const unsigned pos = s_local[dig[e]] + s_runt[dig[e]] + bw + __popc(peers & lanemask_lt());
#pragma unroll
                        for (int w = 0; w < W; ++w) st_k[(size_t)pos * W + w] = key[e].w[w];
                        st_v[pos] = val[e];
                    }
                    __syncthreads();
                    unsigned tot = 0;
#pragma unroll
                    for (int w = 0; w < kOsBlock / 32; ++w) tot += s_w[w][tid];
                    s_runt[tid] += tot;
                    __syncthreads();
                }
                // write out: a bucket's run of the tile to consecutive addresses
                const unsigned len = min((unsigned)kOsTile, n - t0);
                for (unsigned q = tid; q < len; q += kOsBlock) {
                    Key<W> k;
#pragma unroll
                    for (int w = 0; w < W; ++w) k.w[w] = st_k[(size_t)q * W + w];
                    const unsigned bk = sort_digit<W>(k, d);
                    const unsigned long long to = b + s_run[bk] + (q - s_local[bk]);
                    store_key<W>(dk, to, k);
                    dv[to] = st_v[q];
                }
                __syncthreads();
                s_run[tid] += s_cnt[tid];
            }
            __syncthreads();
            half ^= 1;
        }
        if (tid == 0) rot[r].pad = (unsigned)half;
    }
}

// One warp per rotation: the sorted segment's entries added in key order,
// 32 at a time by warp_up_sum (bit for bit the sequential chains of the
// sorted kernels' k_exact_chains), the loads of the next 256 in flight
// meanwhile: the removed |v| into l1 and l2-squared, and (validated
// rotations, sign-tagged entries) the merged radii into arithmetic_l2's
// upper L2 (tpgp_rev.c:734-738 with the non-MPFR upper_l2, :57-62).
__global__ void __launch_bounds__(256) k_hash_xchains(HashArgs a, const unsigned long long* v1,
                                                      const unsigned long long* starts, HashRot* rot) {
    const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const unsigned r = blockIdx.x * 8u + warp;
    if (r >= a.rotations || *reinterpret_cast<volatile unsigned*>(&a.st->status)) return;
    const unsigned long long b = starts[r], e = starts[r + 1];
    const unsigned long long* vals = rot[r].pad ? v1 : a.xlog_vals;
    const bool radii = rot[r].radii != 0;  // warp-uniform
    double l1 = 0.0, sq = 0.0, ar = 0.0;
    unsigned long long nxt[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const unsigned long long i = b + (unsigned long long)q * 32 + lane;
        nxt[q] = i < e ? __ldcg(vals + i) : 0ull;
    }
    for (unsigned long long c = b; c < e; c += 256) {
        unsigned long long cur[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            cur[q] = nxt[q];
            const unsigned long long i = c + 256 + (unsigned long long)q * 32 + lane;
            nxt[q] = i < e ? __ldcg(vals + i) : 0ull;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            if (c + (unsigned long long)q * 32 >= e) break;  // warp-uniform
            const bool has = c + (unsigned long long)q * 32 + lane < e;
            const bool tag = (cur[q] >> 63) != 0ull;
            const double v = from_bits(cur[q] & ~kSignBit);
            const bool rem = has && !tag;
            l1 = warp_up_sum(l1, rem ? v : 0.0, rem, nullptr);
            sq = warp_up_sum(sq, rem ? up_mul(v, v) : 0.0, rem, nullptr);
            if (radii) ar = warp_up_sum(ar, has && tag ? up_mul(v, v) : 0.0, has && tag, nullptr);
        }
    }
    if (lane == 0) {
        rot[r].l1 = l1;
        rot[r].sq = sq;
        rot[r].l2 = sq == 0.0 ? 0.0 : next_up(sqrt(sq));
        rot[r].ar = ar == 0.0 ? 0.0 : next_up(sqrt(ar));
    }
}

// One CTA.  Commits the rotations in order with the checks of
// commit_rotation: table overflow, ENUMERIC (nonfinite merged values), ECAP,
// ledger update, ENUMERIC (ledger), EBUDGET; an empty map is a no-op
// rotation (no ledger change).  The records are staged through shared
// memory in chunks; warp 0 takes them 32 at a time: the term counts by a
// warp scan, the ledger's upward sums by warp_up_sum (the sequential
// chain's bits), each lane's checks on its own prefix, and the rotations
// before the first failing lane commit.  Writes n, ledger, terms_in and status.
constexpr int kChainChunk = 512;
__global__ void __launch_bounds__(256) k_hash_chain(HashArgs a, const HashRot* rot) {
    __shared__ HashRot s_rot[kChainChunk];
    __shared__ int s_stop;
    const unsigned R = a.rotations, lane = threadIdx.x & 31u;
    DeviceState* st = a.st;
    unsigned status = 0;
    unsigned long long n = 0, terms = 0, done = 0;
    Ledger led;
    if (threadIdx.x < 32) {
        status = st->status;
        n = st->n;
        led = st->ledger;
    }
    if (threadIdx.x == 0) s_stop = status != 0;
    const RotParams& p0 = a.ps[0];  // a step's rotations share their options
    for (unsigned base = 0; base < R; base += kChainChunk) {
        __syncthreads();
        if (s_stop) break;
        const unsigned cnt = min((unsigned)kChainChunk, R - base);
        for (unsigned k = threadIdx.x; k < cnt; k += blockDim.x) s_rot[k] = rot[base + k];
        __syncthreads();
        if (threadIdx.x < 32) {
            for (unsigned g = 0; g < cnt && !status; g += 32) {
                const unsigned k = g + lane;
                const bool valid = k < cnt;
                HashRot h{};
                if (valid) h = s_rot[k];
                // terms before and after this rotation
                long long incl = valid ? h.dn : 0ll;
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
                    const long long y = __shfl_up_sync(0xffffffffu, incl, off);
                    if (lane >= (unsigned)off) incl += y;
                }
                const unsigned long long nb = (unsigned long long)((long long)n + incl - h.dn);
                const unsigned long long no = (unsigned long long)((long long)n + incl);
                const bool live = valid && nb != 0;  // an empty map's rotation is a no-op
                double l1i, l2i, sqi, ari;
                warp_up_sum(led.dropped_l1, h.l1, live, &l1i);
                warp_up_sum(led.dropped_l2, h.l2, live, &l2i);
                warp_up_sum(led.dropped_l2_squared, h.sq, live, &sqi);
                warp_up_sum(led.arithmetic_l2, h.ar, live, &ari);  // 0 unless validated
                unsigned f = 0;  // this rotation's failure, in the checks' order
                if (valid) {
                    if (h.flags & ST_TABLE) f = ST_TABLE;
                    else if (h.flags & ST_NUMERIC) f = ST_NUMERIC;
                    else if (!live && h.dn != 0) f = ST_ORDER;  // an empty map cannot gain terms
                    else if (live) {
                        if (p0.max_terms && no > p0.max_terms) f = ST_CAP;
                        else if (!is_finite(l2i) || !is_finite(ari)) f = ST_NUMERIC;
                        else if (p0.max_drop_l2 != 0.0 && l2i > p0.max_drop_l2) f = ST_BUDGET;
                    }
                }
                const unsigned fm = __ballot_sync(0xffffffffu, f != 0);
                const unsigned F = fm ? (unsigned)(__ffs(fm) - 1) : 32u;
                const bool commit = valid && lane < F;
                const unsigned cm = __ballot_sync(0xffffffffu, commit);
                const unsigned lm = __ballot_sync(0xffffffffu, commit && live);
                const unsigned rm = __ballot_sync(0xffffffffu, commit && live && h.removed != 0);
                unsigned long long add = commit ? nb : 0ull, peak = commit && live ? no : 0ull;
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    add += __shfl_xor_sync(0xffffffffu, add, off);
                    peak = max(peak, __shfl_xor_sync(0xffffffffu, peak, off));
                }
                if (cm) {
                    n = __shfl_sync(0xffffffffu, no, 31 - __clz(cm));
                    terms += add;
                    done += __popc(cm);
                }
                if (lm) {
                    const unsigned ll = 31 - __clz(lm);
                    led.dropped_l1 = __shfl_sync(0xffffffffu, l1i, ll);
                    led.dropped_l2 = __shfl_sync(0xffffffffu, l2i, ll);
                    led.dropped_l2_squared = __shfl_sync(0xffffffffu, sqi, ll);
                    led.arithmetic_l2 = __shfl_sync(0xffffffffu, ari, ll);
                    led.rotations += __popc(lm);
                    led.removal_events += __popc(rm);
                    if (peak > led.peak_terms) led.peak_terms = peak;
                    led.arithmetic_enclosed = 0;
                }
                if (fm) status = __shfl_sync(0xffffffffu, f, F);
            }
            if (threadIdx.x == 0) s_stop = status != 0;
        }
    }
    if (threadIdx.x != 0) return;
    // the live count can never exceed the slots claimed (a violated
    // invariant stops the step before the sort reads anything)
    if (!status && n > __ldcg(a.claimed)) status = ST_ORDER;
    if (!status && n > st->out_cap) status = ST_CAPACITY;
    st->status = status;
    st->n_out = 0;  // extraction counter
    if (!status) {
        st->n = n;
        st->ledger = led;
        st->terms_in = terms;
        st->rotations_done = done;
    }
}

// --------------------------------------------------------------- extraction
// Live records of the occupied-slot list, appended with one atomic per warp
// (their order is irrelevant: a sort follows).
template <int W>
__global__ void __launch_bounds__(kHashBlock) k_hash_extract(HashArgs a) {
    if (__ldcg(&a.st->status)) return;
    const unsigned long long len = min(__ldcg(a.claimed), a.slots);
    const unsigned lane = threadIdx.x & 31u;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    // every lane runs the same trip count so the warp ballots stay converged
    const unsigned long long first = (unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u);
    for (unsigned long long base = first; base < len; base += stride) {
        const unsigned long long i = base + lane;
        bool live = false;
        Rec<W> R;
        if (i < len) {
            const Entry<W> E = load_entry<W>(a.occ, i);
            if (E.slot != kNoSlot) {
                R = load_rec<W>(a.rec, E.slot);
                live = R.val != 0ull;
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, live);
        if (!m) continue;
        unsigned long long at = 0;
        if (lane == 0) at = atomicAdd(&a.st->n_out, (unsigned long long)__popc(m));
        at = __shfl_sync(0xffffffffu, at, 0);
        if (live) {
            const unsigned long long pos = at + __popc(m & lanemask_lt());
            store_key<W>(a.ek, pos, R.key);
            a.ev[pos] = R.val;
        }
    }
}

// --------------------------------------------------- CTA-local batched step
// A batched item whose whole step fits in shared memory runs it in one CTA:
// the same pair updates as k_hash_rotate on a shared-memory table, one
// rotation per pass with the commit of k_hash_chain applied after each pass
// (two block barriers per rotation, no global round trips), then a block
// radix sort through the item's global scratch into its output buffer.  An
// item whose table fills up reports ST_TABLE and is re-run on the clustered
// sorted path.
// Per slot: tag, key, two values, and one entry of the occupied-slot list.
template <int W>
constexpr size_t smem_slot_bytes() {
    return 4 + 8 * W + 16 + 4;
}
template <int W>
constexpr unsigned smem_slots_max() {
    return W <= 3 ? 4096u : 2048u;  // tables up to ~200 KB of shared memory
}
constexpr unsigned kSmemSlotsMax = 4096;

template <int W>
__device__ __forceinline__ long long smem_find(const uint32_t* tags, const uint64_t* keys,
                                               unsigned mask, const Key<W>& k, uint32_t skip,
                                               unsigned* empty_at, bool* overflow) {
    unsigned s = (unsigned)hash_of<W>(k) & mask;
    for (unsigned i = 0; i <= mask; ++i) {
        const uint32_t tag = tags[s];
        if (tag == 0u) {
            *empty_at = s;
            return -1;
        }
        if (tag != skip) {
            bool eq = true;
#pragma unroll
            for (int w = 0; w < W; ++w) eq &= keys[(size_t)s * W + w] == k.w[w];
            if (eq) return (long long)s;
        }
        s = (s + 1) & mask;
    }
    *overflow = true;
    return -1;
}

template <int W>
__device__ __forceinline__ long long smem_insert(uint32_t* tags, uint64_t* keys, unsigned mask,
                                                 const Key<W>& k, unsigned from, uint32_t stamp,
                                                 bool* overflow) {
    unsigned s = from;
    for (unsigned i = 0; i <= mask; ++i) {
        if (tags[s] == 0u && atomicCAS(tags + s, 0u, stamp) == 0u) {
#pragma unroll
            for (int w = 0; w < W; ++w) keys[(size_t)s * W + w] = k.w[w];
            return (long long)s;
        }
        s = (s + 1) & mask;
    }
    *overflow = true;
    return -1;
}

template <int W>
__global__ void __launch_bounds__(256) k_batch_hash(const BatchItem* items, const unsigned* ids) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ unsigned long long s_acc[4];
    __shared__ unsigned s_born, s_died, s_removed, s_flags, s_status, s_count;
    __shared__ unsigned long long s_n;
    __shared__ unsigned s_hist[256];
    __shared__ unsigned s_wcnt[8][256];
    const BatchItem& it = items[ids[blockIdx.x]];
    if (!it.active) return;
    const unsigned S = it.table_slots, mask = S - 1u;
    uint64_t* skeys = reinterpret_cast<uint64_t*>(smem_raw);
    unsigned long long* sv[2];
    sv[0] = reinterpret_cast<unsigned long long*>(skeys + (size_t)S * W);
    sv[1] = sv[0] + S;
    uint32_t* stags = reinterpret_cast<uint32_t*>(sv[1] + S);
    unsigned* socc = stags + S;  // occupied slots, in claim order
    __shared__ unsigned s_nocc, s_nocc0;  // count; count when the rotation started
    DeviceState* st = it.scratch.st;
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    for (unsigned k = tid; k < S; k += blockDim.x) {
        stags[k] = 0u;
        sv[0][k] = 0ull;
        sv[1][k] = 0ull;
    }
    if (tid < 4) s_acc[tid] = 0ull;
    if (tid == 0) {
        s_born = s_died = s_removed = s_flags = s_nocc = 0u;
        s_status = st->status;
        s_n = st->n;
    }
    __syncthreads();
    // build from the step's input buffer
    {
        const uint64_t* in_k = it.keys[it.x];
        const double* in_v = it.vals[it.x];
        bool overflow = false;
        for (unsigned long long k = tid; k < s_n; k += blockDim.x) {
            const Key<W> key = load_key<W>(in_k, k);
            const long long slot =
                smem_insert<W>(stags, skeys, mask, key, (unsigned)hash_of<W>(key) & mask, 1u, &overflow);
            if (slot >= 0) {
                sv[0][slot] = dbits(__ldcg(in_v + k));
                socc[atomicAdd(&s_nocc, 1u)] = (unsigned)slot;
            }
        }
        if (overflow) atomicOr(&s_flags, ST_TABLE);
    }
    __syncthreads();
    if (tid == 0) s_nocc0 = s_nocc;
    __syncthreads();
    Ledger led;
    unsigned long long terms = 0;
    if (tid == 0) led = st->ledger;
    for (unsigned r = 0; r < it.rotations; ++r) {
        if (s_status || s_flags) break;  // uniform: read after a barrier
        const RotParams& p = it.ps[r];
        const uint32_t stamp = r + 2u;
        const unsigned long long* vin = sv[r & 1u];
        unsigned long long* vout = sv[(r + 1u) & 1u];
        const Key<W> Q = mask_key<W>(p);
        const double c = p.c, s = p.s;
        PairTally t = empty_tally();
        // one pass over the occupied slots present when the rotation starts
        // (keys it inserts are appended behind them)
        const int top = p.mbit[0];
        const unsigned nocc = s_nocc0;
        for (unsigned k = tid; k < nocc; k += blockDim.x) {
            const unsigned slot = socc[k];
            const unsigned long long vb = vin[slot];
            Key<W> K;
#pragma unroll
            for (int w = 0; w < W; ++w) K.w[w] = skeys[(size_t)slot * W + w];
            bool anti, plus_k, plus_p;
            pair_signs(p, word_at<W>(K, p.i_word), word_at<W>(K, p.j_word), anti, plus_k, plus_p);
            if (!anti) {
                vout[slot] = vb ? settle<W>(p, K, from_bits(vb), true, t) : 0ull;
                continue;
            }
            const Key<W> P = key_xor<W>(K, Q);
            unsigned empty_at = 0;
            bool overflow = false;
            const long long ps = smem_find<W>(stags, skeys, mask, P, stamp, &empty_at, &overflow);
            if (overflow) {
                t.flags |= ST_TABLE;
                continue;
            }
            const unsigned long long pb = ps >= 0 ? vin[ps] : 0ull;
            const bool k_live = vb != 0ull, p_live = pb != 0ull;
            if (!k_live) {
                if (!p_live) vout[slot] = 0ull;
                continue;
            }
            if (p_live && key_bit<W>(K, top)) continue;
            const double v = from_bits(vb);
            double sk = __dmul_rn(v, s);
            if (!plus_k) sk = negate(sk);
            double nk = __dmul_rn(v, c), np = sk;
            if (p_live) {
                const double vp = from_bits(pb);
                double sp = __dmul_rn(vp, s);
                if (!plus_p) sp = negate(sp);
                nk = __dadd_rn(nk, sp);
                np = __dadd_rn(__dmul_rn(vp, c), sk);
            }
            vout[slot] = settle<W>(p, K, nk, true, t);
            const unsigned long long pbits = settle<W>(p, P, np, p_live, t);
            if (ps >= 0) {
                vout[ps] = pbits;
            } else if (pbits) {
                const long long ns = smem_insert<W>(stags, skeys, mask, P, empty_at, stamp, &overflow);
                if (ns >= 0) {
                    vout[ns] = pbits;
                    socc[atomicAdd(&s_nocc, 1u)] = (unsigned)ns;
                } else {
                    t.flags |= ST_TABLE;
                }
            }
        }
        warp_tally(t);
        if (lane == 0) {
            if (t.removed) {
                shared_add_u128(s_acc, t.l1);
                shared_add_u128(s_acc + 2, t.sq);
            }
            if (t.born) atomicAdd(&s_born, t.born);
            if (t.died) atomicAdd(&s_died, t.died);
            if (t.removed) atomicAdd(&s_removed, t.removed);
            if (t.flags) atomicOr(&s_flags, t.flags);
        }
        __syncthreads();
        if (tid == 0) {
            // the commit of k_hash_chain for this rotation
            unsigned status = 0;
            const unsigned long long n = s_n;
            if (s_flags & ST_TABLE) {
                status = ST_TABLE;
            } else if (s_flags & ST_NUMERIC) {
                status = ST_NUMERIC;
            } else if (n > 0) {
                const unsigned long long n_out = n + s_born - s_died;
                if (p.max_terms && n_out > p.max_terms) {
                    status = ST_CAP;
                } else {
                    const double l1 = u128_to_double_up(U128{s_acc[0], s_acc[1]}, p.fx_unit1);
                    const double sq = u128_to_double_up(U128{s_acc[2], s_acc[3]}, p.fx_unit2);
                    const double l2 = sq == 0.0 ? 0.0 : next_up(sqrt(sq));
                    Ledger next = led;
                    next.dropped_l1 = up_add(next.dropped_l1, l1);
                    next.dropped_l2 = up_add(next.dropped_l2, l2);
                    next.dropped_l2_squared = up_add(next.dropped_l2_squared, sq);
                    next.arithmetic_l2 = up_add(next.arithmetic_l2, 0.0);
                    next.rotations += 1;
                    if (s_removed) next.removal_events += 1;
                    if (n_out > next.peak_terms) next.peak_terms = n_out;
                    next.arithmetic_enclosed = 0;
                    if (!is_finite(next.dropped_l2) || !is_finite(next.arithmetic_l2)) {
                        status = ST_NUMERIC;
                    } else if (p.max_drop_l2 != 0.0 && next.dropped_l2 > p.max_drop_l2) {
                        status = ST_BUDGET;
                    } else {
                        led = next;
                        terms += n;
                        s_n = n_out;
                    }
                }
            }
            s_status = status;
            s_acc[0] = s_acc[1] = s_acc[2] = s_acc[3] = 0ull;
            s_born = s_died = s_removed = 0u;
            s_nocc0 = s_nocc;  // this rotation's insertions are done (barrier above)
        }
        __syncthreads();
    }
    // the final values are in sv[rotations & 1]
    const unsigned long long n = s_n;
    if (tid == 0 && !s_status && !s_flags && n > it.scratch.cap) s_status = ST_CAPACITY;
    __syncthreads();
    if (s_status || s_flags) {
        if (tid == 0) st->status = s_status ? s_status : ST_TABLE;
        return;
    }
    // extract live entries into the item's scratch (fk, fv), any order
    const unsigned long long* vf = sv[it.rotations & 1u];
    if (tid == 0) s_count = 0u;
    __syncthreads();
    const unsigned nocc_end = (s_nocc + 31u) & ~31u;  // whole warps for the ballot
    for (unsigned k = tid; k < nocc_end; k += blockDim.x) {
        const unsigned slot = k < s_nocc ? socc[k] : 0u;
        const bool live = k < s_nocc && vf[slot] != 0ull;
        const unsigned m = __ballot_sync(0xffffffffu, live);
        unsigned at = 0;
        if (lane == 0 && m) at = atomicAdd(&s_count, (unsigned)__popc(m));
        at = __shfl_sync(0xffffffffu, at, 0);
        if (live) {
            const unsigned pos = at + __popc(m & lanemask_lt());
            Key<W> K;
#pragma unroll
            for (int w = 0; w < W; ++w) K.w[w] = skeys[(size_t)slot * W + w];
            store_key<W>(it.scratch.fk, pos, K);
            reinterpret_cast<unsigned long long*>(it.scratch.fv)[pos] = vf[slot];
        }
    }
    __syncthreads();
    if (s_count != n) {  // extraction must find exactly the committed count
        if (tid == 0) st->status = ST_ORDER;
        return;
    }
    // stable LSD radix sort (8-bit digits): fk/fv <-> sk/sv, last pass into the output buffer
    const int nd = (int)((it.n_spins + 3) / 4);
    for (int d = 0; d < nd; ++d) {
        const bool from_f = d % 2 == 0;
        const uint64_t* srck = from_f ? it.scratch.fk : it.scratch.sk;
        const unsigned long long* srcv =
            reinterpret_cast<const unsigned long long*>(from_f ? it.scratch.fv : it.scratch.sv);
        uint64_t* dstk = d == nd - 1 ? it.keys[it.y] : (from_f ? it.scratch.sk : it.scratch.fk);
        unsigned long long* dstv = reinterpret_cast<unsigned long long*>(
            d == nd - 1 ? it.vals[it.y] : (from_f ? it.scratch.sv : it.scratch.fv));
        s_hist[tid] = 0u;
        __syncthreads();
        for (unsigned long long i = tid; i < n; i += blockDim.x)
            atomicAdd(&s_hist[sort_digit<W>(load_key<W>(srck, i), d)], 1u);
        __syncthreads();
        // exclusive scan of the 256 counts (one per thread)
        const unsigned mine = s_hist[tid];
        unsigned incl = mine;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= (unsigned)off) incl += y;
        }
        if (lane == 31) s_wcnt[0][warp] = incl;
        __syncthreads();
        unsigned before_w = 0;
        for (unsigned w = 0; w < warp; ++w) before_w += s_wcnt[0][w];
        __syncthreads();
        s_hist[tid] = before_w + incl - mine;  // running base of digit tid
        for (unsigned long long r0 = 0; r0 < n; r0 += blockDim.x) {
            for (int q = lane; q < 256; q += 32) s_wcnt[warp][q] = 0u;
            __syncthreads();
            const unsigned long long i = r0 + tid;
            const bool valid = i < n;
            Key<W> k;
            unsigned long long v = 0;
            unsigned dig = 256;
            if (valid) {
                k = load_key<W>(srck, i);
                v = __ldcg(srcv + i);
                dig = sort_digit<W>(k, d);
            }
            const unsigned peers = __match_any_sync(0xffffffffu, dig);
            if (valid && lane == (unsigned)(__ffs(peers) - 1)) s_wcnt[warp][dig] = __popc(peers);
            __syncthreads();
            if (valid) {
                unsigned before = 0;
                for (unsigned w = 0; w < warp; ++w) before += s_wcnt[w][dig];
                const unsigned long long pos =
                    (unsigned long long)s_hist[dig] + before + __popc(peers & lanemask_lt());
                store_key<W>(dstk, pos, k);
                dstv[pos] = v;
            }
            __syncthreads();
            unsigned tot = 0;
#pragma unroll
            for (int w = 0; w < 8; ++w) tot += s_wcnt[w][tid];
            s_hist[tid] += tot;
            __syncthreads();
        }
    }
    if (tid == 0) {
        st->n = n;
        st->ledger = led;
        st->terms_in = terms;
        st->status = 0u;
    }
}

}  // namespace tg

