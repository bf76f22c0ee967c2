// Sort-free Strang step for the bound ledger: the map lives in an
// open-addressing hash table for the duration of one step, every rotation is
// one pass over the table, and the map is sorted back into the reference
// layout once per step.
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
// Table.  tags[s]: 0 empty, 1 present at step start, r+2 inserted by
// rotation r.  Keys never leave the table during a step (a removed key keeps
// its slot with value 0), so linear probing needs no tombstones: a present
// key is always found before the first empty slot of its probe sequence.
// Values are double-buffered per rotation (read vals[r&1], write
// vals[(r+1)&1]); every occupied slot's new value is written exactly once
// per rotation:
//   commuting key                   -> its own thread
//   pair with at least one live key -> the thread of the smaller live key
//   pair with both keys dead        -> each key's own thread writes 0
//   key inserted by this rotation   -> the inserting thread.
// A key looked up in rotation r is never inserted by another thread in r
// (only its partner inserts it), so probes may skip slots tagged r+2.
//
// Ledger and limits.  Each rotation adds its born/died/removed counts and
// fixed-point sums to per-rotation stat slots; k_hash_chain then applies,
// rotation by rotation on one thread, exactly the commit of
// engine/src/tpgp_rev.c:730-757 (ECAP, ledger, ENUMERIC, EBUDGET), stopping
// at the first failure.  Work after a failing rotation is discarded: the
// step's input map is never written (transactional).
#pragma once
#include "rotate_kernels.cuh"

namespace tg {

constexpr int kHashBlock = 256;
constexpr int kMaxProbe = 2048;  // linear-probe bound; hitting it reports ST_TABLE
constexpr int kStatSlots = 32;   // stat slots per rotation (spreads the atomics)
constexpr int kSortBlock = 256, kSortItems = 8, kSortTile = kSortBlock * kSortItems;

struct HashStat {
    unsigned long long l1_lo, l1_hi, sq_lo, sq_hi;
    unsigned long long born, died, removed;
    unsigned int flags, pad;
};
static_assert(sizeof(HashStat) == 64, "stat slot is one 64-byte line");

struct HashArgs {
    const RotParams* ps;  // the step's rotation list (device)
    unsigned rotations;
    const uint2* runs;    // fused passes: (first rotation, count) per pass
    unsigned passes;      // kernels over the table (= rotations when not fused)
    uint32_t* tags;
    uint64_t* keys;                 // [S][W]
    unsigned long long* vals[2];    // coefficient bit patterns, double-buffered
    unsigned long long slots;       // S (any size: slots are h * S >> 64)
    HashStat* stats;                // [rotations][kStatSlots]
    unsigned long long* claimed;    // slots claimed during the step
    const uint64_t* in_keys;        // the step's input map (never written); its
    const double* in_vals;          // length is st->n when the step starts
    uint64_t* out_keys;             // the step's output map
    double* out_vals;
    unsigned long long out_cap;
    uint64_t* ek;                   // extraction / sort ping-pong buffers, S entries
    unsigned long long* ev;
    uint64_t* tk;
    unsigned long long* tv;
    unsigned* hist;                 // [256][tiles] digit counts, then offsets
    DeviceState* st;
};

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

// Slot of key k (tags other than `skip` compared), or -1 with *empty_at the
// first empty slot of its probe sequence.  *overflow when the probe bound is hit.
template <int W>
__device__ __forceinline__ long long hash_find(const HashArgs& a, const Key<W>& k, uint32_t skip,
                                               unsigned long long* empty_at, bool* overflow) {
    unsigned long long s = slot_of(hash_of<W>(k), a.slots);
    for (int i = 0; i < kMaxProbe; ++i) {
        const uint32_t tag = __ldcg(a.tags + s);
        if (tag == 0) {
            *empty_at = s;
            return -1;
        }
        if (tag != skip && key_eq<W>(load_key<W>(a.keys, s), k)) return (long long)s;
        s = next_slot(s, a.slots);
    }
    *overflow = true;
    return -1;
}

// Claims the first empty slot at or after `from` for k (tag `stamp`).
template <int W>
__device__ __forceinline__ long long hash_insert(const HashArgs& a, const Key<W>& k,
                                                 unsigned long long from, uint32_t stamp,
                                                 bool* overflow) {
    unsigned long long s = from;
    for (int i = 0; i < kMaxProbe; ++i) {
        if (__ldcg(a.tags + s) == 0u && atomicCAS(a.tags + s, 0u, stamp) == 0u) {
            store_key<W>(a.keys, s, k);
            return (long long)s;
        }
        s = next_slot(s, a.slots);
    }
    *overflow = true;
    return -1;
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
template <int W>
__global__ void __launch_bounds__(kHashBlock) k_hash_build(HashArgs a) {
    bool overflow = false;
    unsigned long long claimed = 0;
    const unsigned long long n = __ldcg(&a.st->n);
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long k = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += stride) {
        const Key<W> key = load_key<W>(a.in_keys, k);
        const long long s = hash_insert<W>(a, key, slot_of(hash_of<W>(key), a.slots), 1u, &overflow);
        if (s >= 0) {
            a.vals[0][s] = dbits(__ldcg(a.in_vals + k));
            ++claimed;
        }
    }
    claimed = warp_sum_u64(claimed);
    if ((threadIdx.x & 31) == 0 && claimed) atomicAdd(a.claimed, claimed);
    if (overflow) atomicOr(&a.st->status, ST_TABLE);
}

// --------------------------------------------------------------- rotation
// Per-thread counts (32-bit: a thread handles far fewer than 2^32 slots);
// the removed-weight sums go straight into the CTA's shared 128-bit
// accumulators, which keeps them out of the probe loop's registers.
struct PairTally {
    unsigned born, died, removed, claimed, flags;
};

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
// Returns the bit pattern to store (0 when dropped or removed).  acc: the
// CTA's shared (l1 lo, l1 hi, sq lo, sq hi).
template <int W>
__device__ __forceinline__ unsigned long long settle(const RotParams& p, const Key<W>& key,
                                                     double x, bool was_live, PairTally& t,
                                                     unsigned long long* acc) {
    if (!is_finite(x)) t.flags |= ST_NUMERIC;
    unsigned long long out = dbits(x);
    if (is_zero(x)) {
        out = 0;
    } else if (!key_is_zero<W>(key) && abs_bits(x) <= p.threshold_bits) {
        U128 x1, x2;
        fixed_terms(x, p.fx_unit1, p.fx_unit2, x1, x2);
        shared_add_u128(acc, x1);
        shared_add_u128(acc + 2, x2);
        ++t.removed;
        out = 0;
    }
    if (was_live && !out) ++t.died;
    if (!was_live && out) ++t.born;
    return out;
}

// One rotation over the table (one CTA's share of the slots): each slot's
// tag, value and key are loaded in one round trip, and an anticommuting
// key's first probe loads the probe slot's tag, key and value together.
template <int W, int NT>
__device__ __forceinline__ void hash_pass(const HashArgs& a, unsigned r, unsigned k) {
    constexpr int U = 1;
    __shared__ PairTally s_t[NT / 32];
    __shared__ unsigned long long s_acc[4];  // removed l1 (lo, hi), sq (lo, hi)
    if (threadIdx.x < 4) s_acc[threadIdx.x] = 0ull;
    __syncthreads();
    const RotParams& p = a.ps[r];
    const uint32_t stamp = k + 2u;  // pass k: stamps and buffers; rotation r: parameters
    const unsigned long long* vin = a.vals[k & 1u];
    unsigned long long* vout = a.vals[(k + 1u) & 1u];
    const Key<W> Q = mask_key<W>(p);
    const double c = p.c, s = p.s;
    PairTally t;
    t.born = t.died = t.removed = t.claimed = 0;
    t.flags = 0;
    const unsigned long long S = a.slots;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
         base < S; base += U * stride) {
        // 1. own slots: tag, value and key loaded together
        uint32_t tag[U];
        unsigned long long vb[U];
        Key<W> K[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const unsigned long long slot = base + u * stride;
            tag[u] = 0u;
            vb[u] = 0ull;
            if (slot < S) {
                tag[u] = __ldcg(a.tags + slot);
                vb[u] = __ldcg(vin + slot);
                K[u] = load_key<W>(a.keys, slot);
            }
        }
        // 2. classify; anticommuting keys start their partner probe, again
        //    loading tag, key and value of the probe slot together
        bool act[U], plus_k[U];
        Key<W> P[U], PK[U];
        unsigned long long ps[U], pv[U];
        uint32_t pt[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const unsigned long long slot = base + u * stride;
            act[u] = false;
            if (tag[u] == 0u || tag[u] >= stamp) continue;  // empty, or inserted by this rotation
            bool anti;
            branch_info(p, word_at<W>(K[u], p.i_word), word_at<W>(K[u], p.j_word), anti, plus_k[u]);
            if (!anti) {
                // commuting: merged value v + 0 = v, still subject to the
                // threshold like every merged term (no anticommuting key pairs with it)
                vout[slot] = vb[u] ? settle<W>(p, K[u], from_bits(vb[u]), true, t, s_acc) : 0ull;
                continue;
            }
            act[u] = true;
            P[u] = key_xor<W>(K[u], Q);
            ps[u] = slot_of(hash_of<W>(P[u]), a.slots);
            pt[u] = __ldcg(a.tags + ps[u]);
            PK[u] = load_key<W>(a.keys, ps[u]);
            pv[u] = __ldcg(vin + ps[u]);
        }
        // 3. finish each probe and update the pair
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (!act[u]) continue;
            const unsigned long long slot = base + u * stride;
            long long found = -1;
            unsigned long long empty_at = 0, pb = 0;
            bool overflow = true;
            for (int i = 0; i < kMaxProbe; ++i) {
                if (pt[u] == 0u) {
                    empty_at = ps[u];
                    overflow = false;
                    break;
                }
                if (pt[u] != stamp && key_eq<W>(PK[u], P[u])) {
                    found = (long long)ps[u];
                    pb = pv[u];
                    overflow = false;
                    break;
                }
                ps[u] = next_slot(ps[u], a.slots);
                pt[u] = __ldcg(a.tags + ps[u]);
                PK[u] = load_key<W>(a.keys, ps[u]);
                pv[u] = __ldcg(vin + ps[u]);
            }
            if (overflow) {
                t.flags |= ST_TABLE;
                continue;
            }
            const bool k_live = vb[u] != 0ull, p_live = pb != 0ull;
            if (!k_live) {
                if (!p_live) vout[slot] = 0ull;  // both dead; the partner's thread clears its own
                continue;                        // else the live partner updates the pair
            }
            if (p_live && key_less<W>(P[u], K[u])) continue;  // the smaller live key updates the pair
            bool anti_p, plus_p;
            branch_info(p, word_at<W>(P[u], p.i_word), word_at<W>(P[u], p.j_word), anti_p, plus_p);
            const double v = from_bits(vb[u]);
            double sk = __dmul_rn(v, s);  // K's sin child, landing on P
            if (!plus_k[u]) sk = negate(sk);
            double nk = __dmul_rn(v, c), np = sk;
            if (p_live) {
                const double vp = from_bits(pb);
                double sp = __dmul_rn(vp, s);  // P's sin child, landing on K
                if (!plus_p) sp = negate(sp);
                nk = __dadd_rn(nk, sp);
                np = __dadd_rn(__dmul_rn(vp, c), sk);
            }
            vout[slot] = settle<W>(p, K[u], nk, true, t, s_acc);
            const unsigned long long pbits = settle<W>(p, P[u], np, p_live, t, s_acc);
            if (found >= 0) {
                vout[found] = pbits;
            } else if (pbits) {
                bool ovf = false;
                const long long ns = hash_insert<W>(a, P[u], empty_at, stamp, &ovf);
                if (ns >= 0) {
                    vout[ns] = pbits;
                    ++t.claimed;
                } else {
                    t.flags |= ST_TABLE;
                }
            }
        }
    }
    // block totals, then one set of atomics into this rotation's stat slot
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        t.born += __shfl_down_sync(0xffffffffu, t.born, off);
        t.died += __shfl_down_sync(0xffffffffu, t.died, off);
        t.removed += __shfl_down_sync(0xffffffffu, t.removed, off);
        t.claimed += __shfl_down_sync(0xffffffffu, t.claimed, off);
        t.flags |= __shfl_down_sync(0xffffffffu, t.flags, off);
    }
    if (lane == 0) s_t[warp] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long born = 0, died = 0, removed = 0, claimed = 0;
        unsigned flags = 0;
        for (int w = 0; w < NT / 32; ++w) {
            born += s_t[w].born;
            died += s_t[w].died;
            removed += s_t[w].removed;
            claimed += s_t[w].claimed;
            flags |= s_t[w].flags;
        }
        HashStat* hs = a.stats + (size_t)r * kStatSlots + (blockIdx.x % kStatSlots);
        atomic_add_u128(&hs->l1_lo, &hs->l1_hi, U128{s_acc[0], s_acc[1]});
        atomic_add_u128(&hs->sq_lo, &hs->sq_hi, U128{s_acc[2], s_acc[3]});
        if (born) atomicAdd(&hs->born, born);
        if (died) atomicAdd(&hs->died, died);
        if (removed) atomicAdd(&hs->removed, removed);
        if (claimed) atomicAdd(a.claimed, claimed);
        if (flags) atomicOr(&hs->flags, flags);
    }
}

template <int W>
__global__ void __launch_bounds__(kHashBlock, 4) k_hash_rotate(HashArgs a, unsigned r, unsigned k) {
    hash_pass<W, kHashBlock>(a, r, k);
}

// All rotations of a step in one cooperative launch (one CTA of 1024 threads
// per SM), a bounded grid barrier between rotations; a barrier that gives up
// sets ST_TIMEOUT and the CTA leaves.  The passes are those of k_hash_rotate.
constexpr int kHashPersistentBlock = 1024;
template <int W>
__global__ void __launch_bounds__(kHashPersistentBlock, 1) k_hash_rotate_all(HashArgs a) {
    for (unsigned r = 0; r < a.rotations; ++r) {
        hash_pass<W, kHashPersistentBlock>(a, r, r);
        if (!grid_barrier(a.st)) return;
    }
}

// ------------------------------------------------- fused runs on one site pair
// A run of consecutive rotations on the same two sites (a secular edge's ZZ,
// XX, YY; six at the middle of a Strang step) whose generators span a group
// G of at most four XOR patterns G = {0, b1, b2, b1 ^ b2}.  Every key's coset
// K xor G is closed under each rotation of the run, so each coset is evolved
// on its own through the whole run — per rotation exactly the pair rule of
// hash_pass (commuting members keep v + 0, anticommuting members combine
// with their partner a ^ label(Q)), with the zero drop, threshold and
// removed-weight sums of that rotation — and only the final values are
// written.  The smallest live member's thread evolves a coset; a coset with
// no live member has each member's own thread clear its slot.  Results are
// those of the run's rotations one by one.
constexpr int kMaxRun = 6;

template <int W>
__device__ __forceinline__ void coset_sign(const RotParams& p, const Key<W>& m, bool& anti,
                                           bool& plus) {
    branch_info(p, word_at<W>(m, p.i_word), word_at<W>(m, p.j_word), anti, plus);
}

template <int W>
__global__ void __launch_bounds__(kHashBlock, 2) k_hash_run(HashArgs a, unsigned k) {
    __shared__ unsigned long long s_acc[kMaxRun][4];
    __shared__ unsigned s_cnt[kMaxRun][3];  // born, died, removed
    __shared__ unsigned s_claimed, s_flags;
    for (int q = threadIdx.x; q < kMaxRun * 4; q += blockDim.x) (&s_acc[0][0])[q] = 0ull;
    for (int q = threadIdx.x; q < kMaxRun * 3; q += blockDim.x) (&s_cnt[0][0])[q] = 0u;
    if (threadIdx.x == 0) {
        s_claimed = 0u;
        s_flags = 0u;
    }
    __syncthreads();
    const uint2 run = a.runs[k];
    const unsigned r0 = run.x, L = run.y;
    const uint32_t stamp = k + 2u;
    const unsigned long long* vin = a.vals[k & 1u];
    unsigned long long* vout = a.vals[(k + 1u) & 1u];
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
    unsigned flags = 0u, claimed = 0u;
    const unsigned long long S = a.slots;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long slot = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
         slot < S; slot += stride) {
        const uint32_t tag = __ldcg(a.tags + slot);
        const unsigned long long vb = __ldcg(vin + slot);
        const Key<W> K = load_key<W>(a.keys, slot);
        if (tag == 0u || tag >= stamp) continue;  // empty, or inserted by this pass
        // the coset's other members: first probe slots loaded together
        Key<W> M[4], PK[4];
        unsigned long long ps[4], pv[4], ea[4], v[4];
        uint32_t pt[4];
        long long sl[4];
        M[0] = K;
        sl[0] = (long long)slot;
        v[0] = vb;
        ea[0] = 0ull;
#pragma unroll
        for (int m = 1; m < 4; ++m) {
            M[m] = key_xor<W>(K, G[m]);
            sl[m] = -1;
            v[m] = 0ull;
            ea[m] = 0ull;
            if (m < gs) {
                ps[m] = slot_of(hash_of<W>(M[m]), S);
                pt[m] = __ldcg(a.tags + ps[m]);
                PK[m] = load_key<W>(a.keys, ps[m]);
                pv[m] = __ldcg(vin + ps[m]);
            }
        }
        bool overflow = false;
#pragma unroll
        for (int m = 1; m < 4; ++m) {
            if (m >= gs) continue;
            bool done = false;
            for (int i = 0; i < kMaxProbe; ++i) {
                if (pt[m] == 0u) {
                    ea[m] = ps[m];
                    done = true;
                    break;
                }
                if (pt[m] != stamp && key_eq<W>(PK[m], M[m])) {
                    sl[m] = (long long)ps[m];
                    v[m] = pv[m];
                    done = true;
                    break;
                }
                ps[m] = next_slot(ps[m], S);
                pt[m] = __ldcg(a.tags + ps[m]);
                PK[m] = load_key<W>(a.keys, ps[m]);
                pv[m] = __ldcg(vin + ps[m]);
            }
            if (!done) overflow = true;
        }
        if (overflow) {
            flags |= ST_TABLE;
            continue;
        }
        // the smallest live member evolves the coset
        int h = -1;
#pragma unroll
        for (int m = 0; m < 4; ++m)
            if (m < gs && v[m] && (h < 0 || key_less<W>(M[m], pick<4, Key<W>>(M, h)))) h = m;
        if (h < 0) {
            vout[slot] = 0ull;  // no live member: each member clears its own slot
            continue;
        }
        if (h != 0) continue;
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
            PairTally t;
            t.born = t.died = t.removed = t.claimed = 0u;
            t.flags = 0u;
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                if (!touched[m]) continue;  // absent before and after: no term
                const unsigned long long out = settle<W>(p, M[m], nx[m], live[m], t, s_acc[l]);
                live[m] = out != 0ull;
                x[m] = from_bits(out);
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
                vout[sl[m]] = bits;
            } else if (bits) {
                bool ovf = false;
                const long long ns = hash_insert<W>(a, M[m], ea[m], stamp, &ovf);
                if (ns >= 0) {
                    vout[ns] = bits;
                    ++claimed;
                } else {
                    flags |= ST_TABLE;
                }
            }
        }
    }
    if (flags) atomicOr(&s_flags, flags);
    if (claimed) atomicAdd(&s_claimed, claimed);
    __syncthreads();
    if (threadIdx.x == 0) {
        for (unsigned l = 0; l < L; ++l) {
            HashStat* hs = a.stats + (size_t)(r0 + l) * kStatSlots + (blockIdx.x % kStatSlots);
            atomic_add_u128(&hs->l1_lo, &hs->l1_hi, U128{s_acc[l][0], s_acc[l][1]});
            atomic_add_u128(&hs->sq_lo, &hs->sq_hi, U128{s_acc[l][2], s_acc[l][3]});
            if (s_cnt[l][0]) atomicAdd(&hs->born, (unsigned long long)s_cnt[l][0]);
            if (s_cnt[l][1]) atomicAdd(&hs->died, (unsigned long long)s_cnt[l][1]);
            if (s_cnt[l][2]) atomicAdd(&hs->removed, (unsigned long long)s_cnt[l][2]);
            if (s_flags) atomicOr(&hs->flags, s_flags);
        }
        if (s_claimed) atomicAdd(a.claimed, (unsigned long long)s_claimed);
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
    unsigned flags, pad;
};

__global__ void __launch_bounds__(256) k_hash_reduce(HashArgs a, HashRot* rot) {
    const unsigned r = blockIdx.x * 8u + (threadIdx.x >> 5), lane = threadIdx.x & 31u;
    if (r >= a.rotations) return;
    const HashStat x = a.stats[(size_t)r * kStatSlots + lane];
    U128 l1{x.l1_lo, x.l1_hi}, sq{x.sq_lo, x.sq_hi};
    unsigned long long born = x.born, died = x.died, removed = x.removed;
    unsigned flags = x.flags;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        u128_add(l1, shfl_down_u128(l1, off));
        u128_add(sq, shfl_down_u128(sq, off));
        born += __shfl_down_sync(0xffffffffu, born, off);
        died += __shfl_down_sync(0xffffffffu, died, off);
        removed += __shfl_down_sync(0xffffffffu, removed, off);
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
        rot[r] = h;
    }
}

// One CTA.  Walks the rotations in order on one thread with the commit of
// commit_rotation: table overflow, ENUMERIC (nonfinite merged values), ECAP,
// ledger update, ENUMERIC (ledger), EBUDGET; an empty map is a no-op rotation
// (no ledger change).  The records are staged through shared memory in
// chunks so the sequential walk never waits on global memory.  Writes n,
// ledger, terms_in and status.
constexpr int kChainChunk = 512;
__global__ void __launch_bounds__(256) k_hash_chain(HashArgs a, const HashRot* rot) {
    __shared__ HashRot s_rot[kChainChunk];
    __shared__ int s_stop;
    const unsigned R = a.rotations;
    DeviceState* st = a.st;
    unsigned status = 0;
    unsigned long long n = 0, terms = 0, done = 0;
    Ledger led;
    if (threadIdx.x == 0) {
        status = st->status;
        n = st->n;
        led = st->ledger;
        s_stop = status != 0;
    }
    const RotParams& p0 = a.ps[0];  // a step's rotations share their options
    for (unsigned base = 0; base < R; base += kChainChunk) {
        __syncthreads();
        if (s_stop) break;
        const unsigned cnt = min((unsigned)kChainChunk, R - base);
        for (unsigned k = threadIdx.x; k < cnt; k += blockDim.x) s_rot[k] = rot[base + k];
        __syncthreads();
        if (threadIdx.x == 0) {
            for (unsigned k = 0; k < cnt && !status; ++k) {
                const HashRot& h = s_rot[k];
                if (h.flags & ST_TABLE) {
                    status = ST_TABLE;
                    break;
                }
                if (h.flags & ST_NUMERIC) {
                    status = ST_NUMERIC;
                    break;
                }
                if (n == 0) {  // empty map: the rotation is a no-op
                    ++done;
                    continue;
                }
                const unsigned long long n_out = (unsigned long long)((long long)n + h.dn);
                if (p0.max_terms && n_out > p0.max_terms) {
                    status = ST_CAP;
                    break;
                }
                Ledger next = led;
                next.dropped_l1 = up_add(next.dropped_l1, h.l1);
                next.dropped_l2 = up_add(next.dropped_l2, h.l2);
                next.dropped_l2_squared = up_add(next.dropped_l2_squared, h.sq);
                next.arithmetic_l2 = up_add(next.arithmetic_l2, 0.0);
                next.rotations += 1;
                if (h.removed) next.removal_events += 1;
                if (n_out > next.peak_terms) next.peak_terms = n_out;
                next.arithmetic_enclosed = 0;
                if (!is_finite(next.dropped_l2) || !is_finite(next.arithmetic_l2)) {
                    status = ST_NUMERIC;
                    break;
                }
                if (p0.max_drop_l2 != 0.0 && next.dropped_l2 > p0.max_drop_l2) {
                    status = ST_BUDGET;
                    break;
                }
                led = next;
                terms += n;
                n = n_out;
                ++done;
            }
            s_stop = status != 0;
        }
    }
    if (threadIdx.x != 0) return;
    // the live count can never exceed the slots claimed (a violated
    // invariant stops the step before the sort reads anything)
    if (!status && n > __ldcg(a.claimed)) status = ST_ORDER;
    if (!status && n > a.out_cap) status = ST_CAPACITY;
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
// Live slots of the final value buffer, in slot order per warp, appended
// with one atomic per warp (their order is irrelevant: a sort follows).
template <int W>
__global__ void __launch_bounds__(kHashBlock) k_hash_extract(HashArgs a) {
    if (__ldcg(&a.st->status)) return;
    const unsigned long long* vf = a.vals[a.passes & 1u];
    const unsigned long long S = a.slots;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    // every lane runs the same trip count so the warp ballots stay converged
    const unsigned long long first = (unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u);
    for (unsigned long long base = first; base < S; base += stride) {
        const unsigned long long slot = base + lane;
        bool live = false;
        unsigned long long vb = 0;
        if (slot < S && __ldcg(a.tags + slot) != 0u) {
            vb = __ldcg(vf + slot);
            live = vb != 0ull;
        }
        const unsigned m = __ballot_sync(0xffffffffu, live);
        if (!m) continue;
        unsigned long long at = 0;
        if (lane == 0) at = atomicAdd(&a.st->n_out, (unsigned long long)__popc(m));
        at = __shfl_sync(0xffffffffu, at, 0);
        if (live) {
            const unsigned long long pos = at + __popc(m & lanemask_lt());
            store_key<W>(a.ek, pos, load_key<W>(a.keys, slot));
            a.ev[pos] = vb;
        }
    }
}

// --------------------------------------------------------------- radix sort
// Stable LSD radix sort of the extracted (key, value) pairs by key, 8-bit
// digits from the least significant; the last pass writes the output map.
template <int W>
__device__ __forceinline__ unsigned digit_of(const Key<W>& k, int d) {
    return (unsigned)((word_at<W>(k, d >> 3) >> ((d & 7) * 8)) & 0xffull);
}

template <int W>
__global__ void __launch_bounds__(kSortBlock) k_radix_hist(const uint64_t* keys, HashArgs a,
                                                           int d) {
    __shared__ unsigned cnt[256];
    if (__ldcg(&a.st->status)) return;
    const unsigned long long n = min(__ldcg(&a.st->n), a.slots);  // never beyond the buffers
    if (d == 0 && blockIdx.x == 0 && threadIdx.x == 0 && __ldcg(&a.st->n_out) != n)
        atomicOr(&a.st->status, ST_ORDER);  // extraction must find exactly the committed count
    const unsigned long long ntiles = (n + kSortTile - 1) / kSortTile;
    for (unsigned long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        cnt[threadIdx.x] = 0;
        __syncthreads();
#pragma unroll
        for (int e = 0; e < kSortItems; ++e) {
            const unsigned long long i = tile * kSortTile + (unsigned long long)e * kSortBlock + threadIdx.x;
            if (i < n) atomicAdd(&cnt[digit_of<W>(load_key<W>(keys, i), d)], 1u);
        }
        __syncthreads();
        a.hist[(size_t)threadIdx.x * ntiles + tile] = cnt[threadIdx.x];
        __syncthreads();
    }
}

// Exclusive scan of the digit-major histogram (one CTA of 1024 threads).
__global__ void __launch_bounds__(1024) k_radix_scan(HashArgs a) {
    __shared__ unsigned long long s_part[1024];
    if (__ldcg(&a.st->status)) return;
    const unsigned long long n = min(__ldcg(&a.st->n), a.slots);  // never beyond the buffers
    const unsigned long long total = 256ull * ((n + kSortTile - 1) / kSortTile);
    const unsigned long long per = (total + blockDim.x - 1) / blockDim.x;
    const unsigned long long lo = min(total, per * threadIdx.x), hi = min(total, lo + per);
    unsigned long long sum = 0;
    for (unsigned long long i = lo; i < hi; ++i) sum += a.hist[i];
    s_part[threadIdx.x] = sum;
    __syncthreads();
    for (unsigned off = 1; off < blockDim.x; off <<= 1) {
        const unsigned long long v = threadIdx.x >= off ? s_part[threadIdx.x - off] : 0ull;
        __syncthreads();
        s_part[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned long long run = s_part[threadIdx.x] - sum;
    for (unsigned long long i = lo; i < hi; ++i) {
        const unsigned c = a.hist[i];
        a.hist[i] = (unsigned)run;
        run += c;
    }
}

// Stable scatter: within a tile, elements are ranked in tile order (rounds
// of 256 consecutive elements; within a round by warp, then by lane).
template <int W>
__global__ void __launch_bounds__(kSortBlock) k_radix_scatter(const uint64_t* sk,
                                                              const unsigned long long* sv,
                                                              uint64_t* dk, unsigned long long* dv,
                                                              HashArgs a, int d) {
    __shared__ unsigned base[256];
    __shared__ unsigned wcnt[kSortBlock / 32][256];
    if (__ldcg(&a.st->status)) return;
    const unsigned long long n = min(__ldcg(&a.st->n), a.slots);  // never beyond the buffers
    const unsigned long long ntiles = (n + kSortTile - 1) / kSortTile;
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (unsigned long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        base[threadIdx.x] = a.hist[(size_t)threadIdx.x * ntiles + tile];
        for (int e = 0; e < kSortItems; ++e) {
            // (the barrier at the end of the previous round separates these
            // writes from that round's reads)
            for (int q = lane; q < 256; q += 32) wcnt[warp][q] = 0;
            __syncthreads();
            const unsigned long long i = tile * kSortTile + (unsigned long long)e * kSortBlock + threadIdx.x;
            const bool valid = i < n;
            Key<W> k;
            unsigned long long v = 0;
            unsigned dig = 256;
            if (valid) {
                k = load_key<W>(sk, i);
                v = __ldcg(sv + i);
                dig = digit_of<W>(k, d);
            }
            const unsigned peers = __match_any_sync(0xffffffffu, dig);
            if (valid && lane == (unsigned)(__ffs(peers) - 1)) wcnt[warp][dig] = __popc(peers);
            __syncthreads();
            if (valid) {
                unsigned before = 0;
                for (unsigned w = 0; w < warp; ++w) before += wcnt[w][dig];
                const unsigned long long pos =
                    (unsigned long long)base[dig] + before + __popc(peers & lanemask_lt());
                store_key<W>(dk, pos, k);
                dv[pos] = v;
            }
            __syncthreads();
            unsigned tot = 0;
#pragma unroll
            for (int w = 0; w < kSortBlock / 32; ++w) tot += wcnt[w][threadIdx.x];
            base[threadIdx.x] += tot;
            __syncthreads();
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
        PairTally t;
        t.born = t.died = t.removed = t.claimed = 0;
        t.flags = 0;
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
                vout[slot] = vb ? settle<W>(p, K, from_bits(vb), true, t, s_acc) : 0ull;
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
            vout[slot] = settle<W>(p, K, nk, true, t, s_acc);
            const unsigned long long pbits = settle<W>(p, P, np, p_live, t, s_acc);
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
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            t.born += __shfl_down_sync(0xffffffffu, t.born, off);
            t.died += __shfl_down_sync(0xffffffffu, t.died, off);
            t.removed += __shfl_down_sync(0xffffffffu, t.removed, off);
            t.flags |= __shfl_down_sync(0xffffffffu, t.flags, off);
        }
        if (lane == 0) {
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
            atomicAdd(&s_hist[digit_of<W>(load_key<W>(srck, i), d)], 1u);
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
                dig = digit_of<W>(k, d);
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

