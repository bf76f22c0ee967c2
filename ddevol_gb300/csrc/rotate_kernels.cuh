// Device-resident rotation of a sorted Pauli map: one secular two-spin
// rotation exp(-i theta Q) P exp(+i theta Q) applied to every term, with
// merging of equal keys, exact-zero removal and threshold truncation.
//
// Reference semantics (DDevol engine/src/tpgp_rev.c:535-771, non-validated):
//   * each term (P, v) gives (P, v) and (P, 0) when P commutes with Q, else
//     (P, RN(v c)) and (P xor Q, sign * RN(v s)) with sign = +1 iff the phase
//     exponent of Q P is 1 (tpgp_rev.c:432-467);
//   * children are stably sorted by key and equal keys summed in that order;
//     an exact zero is dropped silently, the identity key is always kept, and
//     |v| <= threshold is removed into the ledger (tpgp_rev.c:689-729).
//
// GB300 design.  Anticommutation with Q is invariant under multiplication by
// Q, so a flipped child never lands on a commuting key and every output key
// has at most two contributions: its own cos child and its partner's sin
// child.  Their sum RN(x + y) does not depend on order, so the reference's
// stable sort need not be reproduced element by element.  The cos children
// keep the input order (already sorted); only the flipped children need
// sorting, and because XOR with Q changes 2-4 key bits the flipped sequence
// is the input order with segment halves swapped.  The rotation therefore
// runs as four streaming passes over HBM, no general sort:
//
//   k_classify  : ballot anticommutation test per term, block+look-back
//                 compaction of the anticommuting terms into (P xor Q, sign v s)
//                 in input order                                   [P1]
//   k_flip_sort : radix placement of the flipped children by the flipped key
//                 bits: for every mask bit (a radix digit) the segment of
//                 terms sharing all higher bits has its 0-half and 1-half
//                 swapped; the displacement of each child is the sum over
//                 digits, computed from in-tile scans of the digit-boundary
//                 positions plus galloping searches at tile edges       [P2]
//   k_partition : merge-path split points between the cos list and the
//                 sorted flipped list, never separating a key pair   [P3a]
//   k_merge     : merge, combine each key pair, drop zeros, threshold,
//                 look-back compaction of the kept terms, per-tile ledger
//                 partial sums, and the next rotation's classification of
//                 every kept term (its flipped children go straight to the
//                 next k_flip_sort); the last CTA commits the rotation:
//                 ledger update, cap and budget checks             [P3b+P1']
// k_classify runs only for the first rotation of a call.
#pragma once
#include "common.cuh"

namespace tg {

// ------------------------------------------------------------- parameters
struct RotParams {
    int i_word, i_shift, j_word, j_shift;  // word and bit offset of sites i, j
    unsigned qi, qj;
    double c, s;            // host-computed cos/sin (never evaluated on device)
    double threshold;
    unsigned long long threshold_bits;  // bit pattern of threshold (>= 0, finite)
    uint64_t mask[4];       // Q's bits: qi at site i, qj at site j
    int nlev;               // number of mask bits (radix digits), 0..4
    int mbit[4];            // mask bit positions, descending
    int nth;                // distinct digit-boundary thresholds
    int th[8];              // threshold bit positions
    int lev_lo[4], lev_hi[4];  // index in th of mbit[l] and mbit[l] + 1
    int exact_ledger;       // 1: removed values kept in order for a sequential ledger
    int validated;          // 1: children carry error radii from rc, rs (hash-table step only)
    double rc, rs;          // radii of c and s (validated)
    unsigned wait_polls;    // device waits give up after this many polls (0: defaults)
    unsigned index;         // position in the call's rotation list
    int fx_unit1, fx_unit2; // fixed-point units of the bound ledger (see fixed_terms)
    unsigned long long max_terms;
    double max_drop_l2;
    // the next rotation's generator, classified inside this rotation's merge
    int has_next;
    int n_i_word, n_i_shift, n_j_word, n_j_shift;
    unsigned n_qi, n_qj;
    double n_s;
    uint64_t n_mask[4];
};

struct Buffers {
    const uint64_t* in_keys;
    const double* in_vals;
    uint64_t* out_keys;
    double* out_vals;
    uint64_t* fk;                  // flipped children, input order
    double* fv;
    uint64_t* sk;                  // flipped children, key order
    double* sv;
    double* rem;                   // removed |v|, per merge tile in key order (exact ledger)
    unsigned* rem_count;           // removed terms per merge tile
    unsigned long long* splits;    // merge-path split (i, j) per tile boundary
    unsigned long long* partials;  // per-tile fixed-point (l1, sq) sums, 4 words per tile
    unsigned long long* p1_tiles;  // look-back words
    unsigned long long* p3_tiles;
    DeviceState* st;
    unsigned long long cap;        // terms each map / child buffer holds
    // exact ledger of a single map: every rotation's removed |v| in key order
    // is appended to `log` (the tile's place from a third look-back channel,
    // p3r_tiles) and its place recorded in rot_log[p.index]; the sequential
    // sums run after the call (k_exact_chains).  log == nullptr: the sums run
    // in the committing CTA (batched items).
    double* log;
    unsigned long long log_cap;
    unsigned long long* p3r_tiles;
    struct RotLog* rot_log;
};

// One rotation's entry in the exact-ledger log.
struct RotLog {
    unsigned long long off, count;  // its removed |v| in log[off, off + count), key order
    unsigned counted, pad;          // 0: a no-op rotation of an empty map (no ledger change)
};

constexpr int kP1Block = 256, kP1Items = 8, kP1Tile = kP1Block * kP1Items;
// An odd number of items per thread keeps the blocked shared-memory accesses
// (thread t reads elements t*I .. t*I+I-1) free of bank conflicts for
// one-word keys (stride 56 B) and at most 2-way for two-word keys.
constexpr int kP2Block = 256, kP2Items = 7, kP2Tile = kP2Block * kP2Items;
constexpr int kP3Block = 256, kP3Items = 7, kP3Tile = kP3Block * kP3Items;
constexpr int kCommitBlock = 1024;
constexpr int kBlInf = 0x7fff;  // digit-boundary level of element 0
static_assert(kP1Items * (kP1Block / 32) == 64, "P1 row/warp scan assumes 64 entries");


// The CTAs that run a phase for one map: the whole grid (per-kernel path and
// persistent kernel) or the CTAs of one thread-block cluster (batched maps).
struct Grid {
    unsigned cta, ncta;
};
__device__ __forceinline__ Grid whole_grid() { return Grid{blockIdx.x, gridDim.x}; }

// Per-term branch data: anticommutation, phase sign.
__device__ __forceinline__ void branch_info(const RotParams& p, uint64_t wi, uint64_t wj,
                                            bool& anti, bool& plus) {
    const unsigned pi = site_symbol(wi, p.i_shift), pj = site_symbol(wj, p.j_shift);
    anti = anticommutes(p.qi, pi) != anticommutes(p.qj, pj);
    plus = ((phase_exponent(p.qi, pi) + phase_exponent(p.qj, pj)) & 3u) == 1u;
}

template <int W>
__device__ __forceinline__ Key<W> mask_key(const RotParams& p) {
    Key<W> m;
#pragma unroll
    for (int w = 0; w < W; ++w) m.w[w] = p.mask[w];
    return m;
}

// ======================================================================= P1
template <int W>
__device__ void phase_classify(const RotParams& p, const Buffers& b, Grid g) {
    constexpr int NW = kP1Block / 32;
    __shared__ unsigned s_counts[kP1Items * NW];
    __shared__ unsigned long long s_tile, s_base;
    DeviceState* st = b.st;
    if (__ldcg(&st->status)) return;
    const unsigned long long n = __ldcg(&st->n);
    const unsigned long long ntiles = (n + kP1Tile - 1) / kP1Tile;
    if (g.cta >= ntiles) return;  // never needed: fewer tiles than CTAs
    const Key<W> M = mask_key<W>(p);
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_tile = atomicAdd(&st->p1_counter, 1u);
        __syncthreads();
        const unsigned long long tile = s_tile;
        if (tile >= ntiles) break;
        const unsigned long long base_k = tile * kP1Tile;
        bool anti[kP1Items], plus[kP1Items];
        unsigned rank[kP1Items];
        bool bad = false;
#pragma unroll
        for (int e = 0; e < kP1Items; ++e) {
            const unsigned long long k = base_k + (unsigned long long)e * kP1Block + threadIdx.x;
            anti[e] = false;
            plus[e] = false;
            if (k < n) {
                const uint64_t wi = __ldcg(b.in_keys + k * W + p.i_word);
                const uint64_t wj = __ldcg(b.in_keys + k * W + p.j_word);
                branch_info(p, wi, wj, anti[e], plus[e]);
                const double v = __ldcg(b.in_vals + k);
                // the reference rejects any nonfinite raw child (tpgp_rev.c:682-688)
                if (!is_finite(v)) bad = true;
            }
            const unsigned ballot = __ballot_sync(0xffffffffu, anti[e]);
            rank[e] = __popc(ballot & lanemask_lt());
            if (lane == 0) s_counts[e * NW + warp] = __popc(ballot);
        }
        if (bad) atomicOr(&st->status, ST_NUMERIC);
        __syncthreads();
        if (warp == 0) {
            // exclusive scan of the kP1Items*NW row/warp counts (row-major = index order)
            unsigned v0 = s_counts[2 * lane], v1 = s_counts[2 * lane + 1];
            unsigned sum = v0 + v1, incl = sum;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const unsigned t = __shfl_up_sync(0xffffffffu, incl, off);
                if (lane >= (unsigned)off) incl += t;
            }
            const unsigned excl = incl - sum;
            s_counts[2 * lane] = excl;
            s_counts[2 * lane + 1] = excl + v0;
            const unsigned total = __shfl_sync(0xffffffffu, incl, 31);
            const unsigned long long base =
                lookback_exclusive(b.p1_tiles, tile, pack2(total, 0), &st->status,
                                   poll_limit(st, kLookbackPolls));
            if (lane == 0) {
                unsigned long long lo, hi;
                unpack2(base, lo, hi);
                s_base = lo;
                if (tile == ntiles - 1) {
                    const unsigned long long a = lo + total;
                    st->a = a;
                    st->p1_tiles = ntiles;
                    if (n + a > b.cap) atomicOr(&st->status, ST_CAPACITY);
                }
            }
        }
        __syncthreads();
        const unsigned long long base = s_base;
#pragma unroll
        for (int e = 0; e < kP1Items; ++e) {
            if (!anti[e]) continue;
            const unsigned long long k = base_k + (unsigned long long)e * kP1Block + threadIdx.x;
            const unsigned long long x = base + s_counts[e * NW + warp] + rank[e];
            if (x >= b.cap) {
                atomicOr(&st->status, ST_CAPACITY);
                continue;
            }
            const Key<W> key = load_key<W>(b.in_keys, k);
            const double v = __ldcg(b.in_vals + k);
            const double y = __dmul_rn(v, p.s);
            store_key<W>(b.fk, x, key_xor<W>(key, M));
            reinterpret_cast<unsigned long long*>(b.fv)[x] = dbits(y) ^ (plus[e] ? 0ull : kSignBit);
        }
    }
}

template <int W>
__global__ void __launch_bounds__(kP1Block) k_classify(RotParams p, Buffers b) {
    pdl_enter();
    phase_classify<W>(p, b, whole_grid());
}

// ======================================================================= P2
// Warp-cooperative search over the anticommuting sequence A (A[y] = fk[y]
// xor M) for the start of the run of elements that share all bits >= theta
// with A[from] (backward = true), or for the first element after that run
// (forward; a if the run reaches the end).  The predicate is monotone on each
// side of `from`.  Each round the 32 lanes probe 32 positions: spaced by a
// step that grows 32x per round while the run continues, then evenly inside
// the bracketing interval, which shrinks 32x per round; so a run of length L
// costs ~2 log_32(L) dependent loads.  Every lane of the (converged) warp
// calls it and gets the same result.
template <int W>
__device__ unsigned long long run_edge_warp(const uint64_t* fk, const Key<W>& M,
                                            unsigned long long a, unsigned long long from,
                                            int theta, bool backward) {
    const long long lane = (long long)lane_id();
    const Key<W> target = key_high<W>(key_xor<W>(load_key_coherent<W>(fk, from), M), theta);
    auto same = [&](long long y) {
        return key_eq<W>(key_high<W>(key_xor<W>(load_key_coherent<W>(fk, (size_t)y), M), theta),
                         target);
    };
    const long long n = (long long)a;
    if (backward) {
        // smallest y <= from with same(y); bracket (bad, good]: !same(bad) (or bad = -1), same(good)
        long long good = (long long)from, bad = -1, step = 1;
        while (true) {
            const long long y = good - (lane + 1) * step;
            const unsigned fails = __ballot_sync(0xffffffffu, !(y >= 0 && same(y)));
            if (fails) {
                const long long l = __ffs(fails) - 1;
                bad = max(-1ll, good - (l + 1) * step);
                good -= l * step;
                break;
            }
            good -= 32 * step;
            step *= 32;
        }
        while (good - bad > 1) {
            const long long c = good - bad - 1;
            const long long y = c <= 32 ? bad + 1 + lane : bad + 1 + (lane * c) / 32;
            const bool in = lane < c || c > 32;
            const unsigned hits = __ballot_sync(0xffffffffu, in && same(y));
            if (!hits) {
                if (c <= 32) break;
                bad = __shfl_sync(0xffffffffu, y, 31);
            } else {
                const int f = __ffs(hits) - 1;
                const long long yf = __shfl_sync(0xffffffffu, y, f);
                const long long yp = __shfl_sync(0xffffffffu, y, f > 0 ? f - 1 : 0);
                good = yf;
                if (c <= 32) break;
                if (f > 0) bad = yp;
            }
        }
        return (unsigned long long)good;
    }
    // smallest y > from with !same(y), or a; bracket [good, bad): same(good), !same(bad) (or bad = a)
    long long good = (long long)from, bad = n, step = 1;
    while (true) {
        const long long y = good + (lane + 1) * step;
        const unsigned fails = __ballot_sync(0xffffffffu, !(y < n && same(y)));
        if (fails) {
            const long long l = __ffs(fails) - 1;
            bad = min(n, good + (l + 1) * step);
            good += l * step;
            break;
        }
        good += 32 * step;
        step *= 32;
    }
    while (bad - good > 1) {
        const long long c = bad - good - 1;
        const long long y = c <= 32 ? good + 1 + lane : good + 1 + (lane * c) / 32;
        const bool in = lane < c || c > 32;
        const unsigned miss = __ballot_sync(0xffffffffu, in && !same(y));
        if (!miss) {
            if (c <= 32) break;
            good = __shfl_sync(0xffffffffu, y, 31);
        } else {
            const int f = __ffs(miss) - 1;
            const long long yf = __shfl_sync(0xffffffffu, y, f);
            const long long yp = __shfl_sync(0xffffffffu, y, f > 0 ? f - 1 : 0);
            bad = yf;
            if (c <= 32) break;
            if (f > 0) good = yp;
        }
    }
    return (unsigned long long)bad;
}

// NT: compile-time bound on the number of digit-boundary thresholds (4 when
// each site carries one mask bit, 6 otherwise).  Positions inside the kernel
// are 32-bit and relative to the tile start (a map holds < 2^30 terms).
template <int W, int NT>
__device__ void phase_flip(const RotParams& p, const Buffers& b, unsigned char* smem_raw, Grid g) {
    uint64_t* s_keys = reinterpret_cast<uint64_t*>(smem_raw);                 // [tile][W]
    double* s_vals = reinterpret_cast<double*>(s_keys + (size_t)kP2Tile * W);  // [tile]
    short* s_bl = reinterpret_cast<short*>(s_vals + kP2Tile);                 // [tile]
    __shared__ int s_gprev[NT], s_gnext[NT];
    __shared__ int s_wprev[kP2Block / 32][NT], s_wnext[kP2Block / 32][NT];
    constexpr int kNone = INT_MIN, kEnd = INT_MAX;

    DeviceState* st = b.st;
    if (__ldcg(&st->status)) return;
    const unsigned long long a = __ldcg(&st->a);
    if (a == 0 || p.nlev == 0) return;
    const unsigned long long ntiles = (a + kP2Tile - 1) / kP2Tile;
    const Key<W> M = mask_key<W>(p);
    const int nth = p.nth;
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    int th[NT];
#pragma unroll
    for (int q = 0; q < NT; ++q) th[q] = q < nth ? p.th[q] : 0x7fffffff;  // unused: never reached

    for (unsigned long long tile = g.cta; tile < ntiles; tile += g.ncta) {
        const unsigned long long x0 = tile * kP2Tile;
        const int len = (int)((a - x0) < (unsigned long long)kP2Tile ? (a - x0) : (unsigned long long)kP2Tile);
        const unsigned long long x1 = x0 + len;
        __syncthreads();
        for (int e = threadIdx.x; e < len; e += kP2Block) {
            const Key<W> k = load_key<W>(b.fk, x0 + e);
#pragma unroll
            for (int w = 0; w < W; ++w) s_keys[(size_t)e * W + w] = k.w[w];
            s_vals[e] = __ldcg(b.fv + x0 + e);
        }
        // run edges outside the tile for every threshold (one warp per
        // search), as offsets from x0
        for (int sq = (int)warp; sq < 2 * nth; sq += kP2Block / 32) {
            const int q = sq % nth;
            if (sq < nth) {
                // last y < x0 with bl(y) >= th[q]: start of the run holding x0-1
                const long long r =
                    x0 == 0 ? 0 : (long long)run_edge_warp<W>(b.fk, M, a, x0 - 1, p.th[q], true);
                if (lane == 0) s_gprev[q] = x0 == 0 ? kNone : (int)(r - (long long)x0);
            } else {
                // first y >= x1 with bl(y) >= th[q] (a if none)
                const unsigned long long g =
                    x1 >= a ? a : max(x1, run_edge_warp<W>(b.fk, M, a, x1 - 1, p.th[q], false));
                if (lane == 0) s_gnext[q] = (int)((long long)g - (long long)x0);
            }
        }
        __syncthreads();
        // digit-boundary level of each element: highest bit differing from its predecessor
        for (int e = threadIdx.x; e < len; e += kP2Block) {
            int bl;
            const unsigned long long x = x0 + e;
            if (x == 0) {
                bl = kBlInf;
            } else {
                Key<W> cur, prev;
#pragma unroll
                for (int w = 0; w < W; ++w) cur.w[w] = s_keys[(size_t)e * W + w];
                if (e > 0) {
#pragma unroll
                    for (int w = 0; w < W; ++w) prev.w[w] = s_keys[(size_t)(e - 1) * W + w];
                } else {
                    prev = load_key<W>(b.fk, x - 1);
                }
                bl = highest_diff_bit<W>(cur, prev);
            }
            s_bl[e] = (short)bl;
        }
        __syncthreads();

        // blocked ownership: thread t owns tile elements [t*I, t*I + I)
        const int e0 = threadIdx.x * kP2Items;
        int lprev[NT], lnext[NT];
#pragma unroll
        for (int q = 0; q < NT; ++q) {
            lprev[q] = kNone;
            lnext[q] = kEnd;
        }
        int blv[kP2Items];
#pragma unroll
        for (int e = 0; e < kP2Items; ++e) {
            const int te = e0 + e;
            blv[e] = te < len ? s_bl[te] : -1;
#pragma unroll
            for (int q = 0; q < NT; ++q) {
                if (blv[e] >= th[q]) {
                    lprev[q] = te;
                    if (lnext[q] == kEnd) lnext[q] = te;
                }
            }
        }
        // exclusive cross-thread scans: max of earlier threads' last, min of later threads' first
        int cprev[NT], cnext[NT];
#pragma unroll
        for (int q = 0; q < NT; ++q) {
            int incl = lprev[q];
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, off);
                if (lane >= (unsigned)off) incl = max(incl, t);
            }
            int excl = __shfl_up_sync(0xffffffffu, incl, 1);
            if (lane == 0) excl = kNone;
            cprev[q] = excl;
            if (lane == 31) s_wprev[warp][q] = incl;
            int rincl = lnext[q];
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int t = __shfl_down_sync(0xffffffffu, rincl, off);
                if (lane + off < 32) rincl = min(rincl, t);
            }
            int rexcl = __shfl_down_sync(0xffffffffu, rincl, 1);
            if (lane == 31) rexcl = kEnd;
            cnext[q] = rexcl;
            if (lane == 0) s_wnext[warp][q] = rincl;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < NT; ++q) {
            int pv = kNone, nv = kEnd;
            for (int w = 0; w < (int)warp; ++w) pv = max(pv, s_wprev[w][q]);
            for (int w = (int)warp + 1; w < kP2Block / 32; ++w) nv = min(nv, s_wnext[w][q]);
            cprev[q] = max(cprev[q], pv);
            cnext[q] = min(cnext[q], nv);
            if (q < nth) {
                if (cprev[q] == kNone) cprev[q] = s_gprev[q];
                if (cnext[q] == kEnd) cnext[q] = s_gnext[q];
            }
        }
        // digits of each element (original key bit = flipped bit xor 1) and
        // displacement: forward pass moves 1-digits back by n0, backward
        // pass moves 0-digits ahead by n1
        int disp[kP2Items];
        {
            int run[NT];
#pragma unroll
            for (int q = 0; q < NT; ++q) run[q] = cprev[q];
#pragma unroll
            for (int e = 0; e < kP2Items; ++e) {
                const int te = e0 + e;
                disp[e] = 0;
                if (te >= len) continue;
#pragma unroll
                for (int q = 0; q < NT; ++q)
                    if (blv[e] >= th[q]) run[q] = te;
                Key<W> fkey;
#pragma unroll
                for (int w = 0; w < W; ++w) fkey.w[w] = s_keys[(size_t)te * W + w];
#pragma unroll
                for (int l = 0; l < 4; ++l) {
                    if (l >= p.nlev) break;
                    if (key_bit<W>(fkey, p.mbit[l]) == 0) {  // original digit 1
                        const int sp = pick<NT>(run, p.lev_lo[l]), sg = pick<NT>(run, p.lev_hi[l]);
                        disp[e] -= (sp == sg) ? 0 : (sp - sg);
                    }
                }
            }
        }
        {
            int run[NT];
#pragma unroll
            for (int q = 0; q < NT; ++q) run[q] = cnext[q];
#pragma unroll
            for (int e = kP2Items - 1; e >= 0; --e) {
                const int te = e0 + e;
                if (te >= len) continue;
                Key<W> fkey;
#pragma unroll
                for (int w = 0; w < W; ++w) fkey.w[w] = s_keys[(size_t)te * W + w];
#pragma unroll
                for (int l = 0; l < 4; ++l) {
                    if (l >= p.nlev) break;
                    if (key_bit<W>(fkey, p.mbit[l]) == 1) {  // original digit 0
                        const int sp = pick<NT>(run, p.lev_lo[l]), en = pick<NT>(run, p.lev_hi[l]);
                        disp[e] += (sp == en) ? 0 : (en - sp);
                    }
                }
                const long long dest = (long long)x0 + te + disp[e];
                if (dest >= 0 && (unsigned long long)dest < a) {
                    store_key<W>(b.sk, (unsigned long long)dest, fkey);
                    b.sv[dest] = s_vals[te];
                } else {
                    atomicOr(&st->status, ST_ORDER);
                }
#pragma unroll
                for (int q = 0; q < NT; ++q)
                    if (blv[e] >= th[q]) run[q] = te;
            }
        }
    }
}

template <int W, int NT>
__global__ void __launch_bounds__(kP2Block) k_flip_sort(RotParams p, Buffers b) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    pdl_enter();
    phase_flip<W, NT>(p, b, smem_raw, whole_grid());
}

// ====================================================================== P3a
// One warp per tile boundary: a 32-ary search along the merge-path diagonal
// (each round the 32 lanes probe 32 evenly spaced positions in parallel), so
// a split costs ~log_32(n) dependent memory round trips instead of log_2(n).
template <int W>
__device__ void phase_partition(const RotParams& p, const Buffers& b, Grid g) {
    DeviceState* st = b.st;
    if (__ldcg(&st->status)) return;
    const unsigned long long n = __ldcg(&st->n), a = __ldcg(&st->a), L = n + a;
    const unsigned long long ntiles = (L + kP3Tile - 1) / kP3Tile;
    const unsigned lane = lane_id();
    const unsigned long long warps = (unsigned long long)g.ncta * (blockDim.x / 32);
    for (unsigned long long t = (unsigned long long)g.cta * (blockDim.x / 32) + (threadIdx.x >> 5);
         t <= ntiles; t += warps) {
        const unsigned long long d = min(t * (unsigned long long)kP3Tile, L);
        // smallest i in [lo, hi] with K[i] merged after S[d-i-1] (ties: cos list first)
        unsigned long long lo = d > a ? d - a : 0, hi = min(d, n);
        while (hi > lo) {
            const unsigned long long span = hi - lo;
            const unsigned long long step = span <= 32 ? 1 : (span + 31) / 32;
            const unsigned long long probe = lo + (unsigned long long)(lane + 1) * step - 1;
            bool before = false;
            if (probe < hi)
                before = key_le<W>(load_key<W>(b.in_keys, probe), load_key<W>(b.sk, d - probe - 1));
            const unsigned c = __popc(__ballot_sync(0xffffffffu, before));
            const unsigned long long new_lo = lo + (unsigned long long)c * step;
            const unsigned long long new_hi = min(hi, lo + (unsigned long long)(c + 1) * step - 1);
            if (step == 1) {
                lo = new_lo;
                break;
            }
            lo = new_lo;
            hi = max(new_lo, new_hi);
        }
        if (lane == 0) {
            unsigned long long i = lo, j = d - lo;
            // keep a (cos, sin) pair with equal keys inside one tile
            if (i > 0 && j < a && key_eq<W>(load_key<W>(b.in_keys, i - 1), load_key<W>(b.sk, j))) ++j;
            b.splits[2 * t] = i;
            b.splits[2 * t + 1] = j;
        }
    }
}

template <int W>
__global__ void k_partition(RotParams p, Buffers b) {
    pdl_enter();
    phase_partition<W>(p, b, whole_grid());
}

// ====================================================================== P3b
// Merge + combine + threshold + compaction of rotation r, fused with the
// classification of rotation r+1 (when p.has_next): every kept output term
// is tested against the next generator and, if it anticommutes, its flipped
// child is written straight into fk/fv for the next rotation's k_flip_sort,
// so the map is read once per rotation.  The look-back word carries
// (kept, next-anticommuting) counts.  The last CTA to finish commits the
// rotation (ledger, cap, budget) and resets the per-rotation state.

// Ledger update of tpgp_rev.c:730-753 (non-validated) by one CTA, then the
// per-rotation reset.  Fields written by other CTAs are read with __ldcg.
template <int NT>
__device__ void commit_rotation(const RotParams& p, const Buffers& b, unsigned long long ntiles) {
    constexpr int NW = NT / 32;
    constexpr unsigned long long T = kP3Tile + 1;
    __shared__ U128 c_l1[NW], c_sq[NW];
    __shared__ unsigned long long c_n, c_a;
    __shared__ unsigned c_status;
    DeviceState* st = b.st;
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        c_status = __ldcg(&st->status);
        c_n = __ldcg(&st->n);
        c_a = __ldcg(&st->a);
    }
    __syncthreads();
    const unsigned status = c_status;
    const unsigned long long n = c_n;
    double l1 = 0.0, sq = 0.0;
    const bool logged = p.exact_ledger && b.log;
    if (!status && n > 0) {
        if (logged) {
            // the sums run after the call; record where this rotation's values are
            if (threadIdx.x == 0) {
                const unsigned long long pos = __ldcg(&st->log_pos), cnt = __ldcg(&st->removed);
                if (pos + cnt > b.log_cap) {
                    atomicOr(&st->status, ST_LOG);
                    st->log_need = pos + cnt;
                } else {
                    b.rot_log[p.index] = RotLog{pos, cnt, 1u, 0u};
                    st->log_pos = pos + cnt;
                }
            }
        } else if (p.exact_ledger) {
            // the reference's sequential order: key order = tile order, one thread
            if (threadIdx.x == 0) {
                for (unsigned long long t = 0; t < ntiles; ++t) {
                    const unsigned cnt = __ldcg(b.rem_count + t);
                    const double* r = b.rem + t * T;
                    for (unsigned k = 0; k < cnt; ++k) {
                        const double v = __ldcg(r + k);
                        l1 = up_add(l1, v);
                        sq = up_add(sq, up_mul(v, v));
                    }
                }
            }
        } else {
            // exact 128-bit sums of the per-tile fixed-point partials, then
            // one upward conversion each
            U128 a1{0ull, 0ull}, a2{0ull, 0ull};
            for (unsigned long long t = threadIdx.x; t < ntiles; t += NT) {
                u128_add(a1, U128{__ldcg(b.partials + 4 * t), __ldcg(b.partials + 4 * t + 1)});
                u128_add(a2, U128{__ldcg(b.partials + 4 * t + 2), __ldcg(b.partials + 4 * t + 3)});
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                u128_add(a1, shfl_down_u128(a1, off));
                u128_add(a2, shfl_down_u128(a2, off));
            }
            if (lane == 0) {
                c_l1[warp] = a1;
                c_sq[warp] = a2;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                U128 t1{0ull, 0ull}, t2{0ull, 0ull};
                for (int w = 0; w < NW; ++w) {
                    u128_add(t1, c_l1[w]);
                    u128_add(t2, c_sq[w]);
                }
                l1 = u128_to_double_up(t1, p.fx_unit1);
                sq = u128_to_double_up(t2, p.fx_unit2);
            }
        }
        if (threadIdx.x == 0) {
            const unsigned long long n_out = __ldcg(&st->n_out);
            const unsigned long long removed = __ldcg(&st->removed);
            unsigned fail = 0;
            if (p.max_terms && n_out > p.max_terms) fail = ST_CAP;
            Ledger next;
            next.dropped_l1 = __ldcg(&st->ledger.dropped_l1);
            next.dropped_l2 = __ldcg(&st->ledger.dropped_l2);
            next.dropped_l2_squared = __ldcg(&st->ledger.dropped_l2_squared);
            next.arithmetic_l2 = __ldcg(&st->ledger.arithmetic_l2);
            next.rotations = __ldcg(&st->ledger.rotations);
            next.removal_events = __ldcg(&st->ledger.removal_events);
            next.peak_terms = __ldcg(&st->ledger.peak_terms);
            next.arithmetic_enclosed = __ldcg(&st->ledger.arithmetic_enclosed);
            if (!fail && __ldcg(&st->status) & ST_LOG) fail = ST_LOG;
            if (!fail) {
                if (!logged) {
                    const double l2 = sq == 0.0 ? 0.0 : next_up(sqrt(sq));
                    next.dropped_l1 = up_add(next.dropped_l1, l1);
                    next.dropped_l2 = up_add(next.dropped_l2, l2);
                    next.dropped_l2_squared = up_add(next.dropped_l2_squared, sq);
                    next.arithmetic_l2 = up_add(next.arithmetic_l2, 0.0);
                }
                next.rotations += 1;
                if (removed) next.removal_events += 1;
                if (n_out > next.peak_terms) next.peak_terms = n_out;
                next.arithmetic_enclosed = 0;
                // with the log, the removed-weight sums and their checks
                // (ENUMERIC, EBUDGET) follow in rotation order after the call
                if (!logged) {
                    if (!is_finite(next.dropped_l2) || !is_finite(next.arithmetic_l2)) fail = ST_NUMERIC;
                    else if (p.max_drop_l2 != 0.0 && next.dropped_l2 > p.max_drop_l2) fail = ST_BUDGET;
                }
            }
            if (fail) {
                atomicOr(&st->status, fail);
            } else {
                st->ledger = next;
                st->n = n_out;
                st->a = p.has_next ? __ldcg(&st->a_next) : 0;
                st->rotations_done = __ldcg(&st->rotations_done) + 1;
                st->terms_in = __ldcg(&st->terms_in) + n;
            }
        }
    } else if (!status && threadIdx.x == 0) {
        st->rotations_done = __ldcg(&st->rotations_done) + 1;  // empty map: no-op, no ledger change
        st->a = 0;
        if (logged) b.rot_log[p.index] = RotLog{0ull, 0ull, 0u, 0u};
    }
    __syncthreads();
    // clear the look-back words this rotation used (clamped to the arrays)
    const unsigned long long t1_max = (b.cap + kP1Tile - 1) / kP1Tile;
    const unsigned long long t3_max = (b.cap + kP3Tile - 1) / kP3Tile;
    const unsigned long long t1 = min((n + kP1Tile - 1) / kP1Tile, t1_max);
    const unsigned long long t3 = min(ntiles, t3_max);
    for (unsigned long long t = threadIdx.x; t <= t1; t += NT) b.p1_tiles[t] = 0;
    for (unsigned long long t = threadIdx.x; t <= t3; t += NT) b.p3_tiles[t] = 0;
    if (logged)
        for (unsigned long long t = threadIdx.x; t <= t3; t += NT) b.p3r_tiles[t] = 0;
    if (threadIdx.x == 0) {
        st->p1_counter = 0;
        st->p3_counter = 0;
        st->merge_done = 0;
        st->n_out = 0;
        st->removed = 0;
        st->a_next = 0;
        // read by every CTA of the persistent kernel after the next barrier
        st->stop = __ldcg(&st->status) != 0 ? 1u : 0u;
    }
    (void)c_a;
}

// every_cta: all CTAs of the grid run this phase (persistent kernel), so all
// of them take part in electing the committing CTA; otherwise only the CTAs
// that can find a tile take part.
template <int W>
__device__ void phase_merge(const RotParams& p, const Buffers& b, unsigned char* smem_raw,
                            bool every_cta, Grid g) {
    constexpr int T = kP3Tile + 1;  // one extra slot for a pair moved across the boundary
    constexpr int NW = kP3Block / 32;
    uint64_t* s_kk = reinterpret_cast<uint64_t*>(smem_raw);       // cos-list keys [T][W]
    uint64_t* s_fk = s_kk + (size_t)T * W;                        // sorted flipped keys
    double* s_kv = reinterpret_cast<double*>(s_fk + (size_t)T * W);
    double* s_fv = s_kv + T;
    __shared__ unsigned long long s_tile, s_base_k, s_base_n, s_base_r;
    __shared__ unsigned s_wk[NW], s_wn[NW], s_wr[NW];
    __shared__ U128 s_l1[NW], s_sq[NW];
    __shared__ int s_last;

    DeviceState* st = b.st;
    // in the persistent kernel every CTA must reach the commit election even
    // after a failure, so a set status only skips the tile work
    const bool failed = *reinterpret_cast<volatile unsigned*>(&st->status) != 0;
    if (failed && !every_cta) return;
    const unsigned long long n = __ldcg(&st->n), a = __ldcg(&st->a), L = n + a;
    const unsigned long long ntiles = failed ? 0 : (L + kP3Tile - 1) / kP3Tile;
    const unsigned long long participants =
        every_cta ? (unsigned long long)g.ncta : max(1ull, min((unsigned long long)g.ncta, ntiles));
    if (g.cta >= participants) return;
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    const double c = p.c;
    Key<W> MN;
#pragma unroll
    for (int w = 0; w < W; ++w) MN.w[w] = p.n_mask[w];
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_tile = atomicAdd(&st->p3_counter, 1u);
        __syncthreads();
        const unsigned long long tile = s_tile;
        if (tile >= ntiles) break;
        const unsigned long long i0 = __ldcg(b.splits + 2 * tile), j0 = __ldcg(b.splits + 2 * tile + 1);
        const unsigned long long i1 = __ldcg(b.splits + 2 * tile + 2), j1 = __ldcg(b.splits + 2 * tile + 3);
        int nk = (int)(i1 - i0), nf = (int)(j1 - j0);
        // the split points guarantee 0 <= nk, nf and nk + nf <= T; a tile that
        // breaks this is flagged and processed as empty (it still publishes
        // its look-back word, so later tiles never wait on it)
        if (i1 < i0 || j1 < j0 || i1 > n || j1 > a || (i1 - i0) + (j1 - j0) > (unsigned long long)T) {
            if (threadIdx.x == 0) atomicOr(&st->status, ST_ORDER);
            nk = 0;
            nf = 0;
        }
        const int len = nk + nf;
        for (int e = threadIdx.x; e < nk; e += kP3Block) {
            const Key<W> k = load_key<W>(b.in_keys, i0 + e);
#pragma unroll
            for (int w = 0; w < W; ++w) s_kk[(size_t)e * W + w] = k.w[w];
            s_kv[e] = __ldcg(b.in_vals + i0 + e);
        }
        for (int e = threadIdx.x; e < nf; e += kP3Block) {
            const Key<W> k = load_key<W>(b.sk, j0 + e);
#pragma unroll
            for (int w = 0; w < W; ++w) s_fk[(size_t)e * W + w] = k.w[w];
            s_fv[e] = __ldcg(b.sv + j0 + e);
        }
        __syncthreads();
        auto kkey = [&](int e) {
            Key<W> k;
#pragma unroll
            for (int w = 0; w < W; ++w) k.w[w] = s_kk[(size_t)e * W + w];
            return k;
        };
        auto fkey = [&](int e) {
            Key<W> k;
#pragma unroll
            for (int w = 0; w < W; ++w) k.w[w] = s_fk[(size_t)e * W + w];
            return k;
        };
        // each thread merges its own output range [lo_d, hi_d) in registers:
        // merge-path split in shared memory, then a serial merge where a cos
        // child absorbs its sin partner (the next merged element, equal key)
        // and a sin child that follows its partner is skipped
        const int lo_d = min(len, (int)threadIdx.x * kP3Items);
        const int hi_d = threadIdx.x == kP3Block - 1 ? len : min(len, lo_d + kP3Items);
        int ik, jf;
        {
            int lo = max(0, lo_d - nf), hi = min(lo_d, nk);
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (key_le<W>(kkey(mid), fkey(lo_d - mid - 1))) lo = mid + 1;
                else hi = mid;
            }
            ik = lo;
            jf = lo_d - lo;
        }
        // classify: 0 drop, 1 keep, 2 removed; nx: kept and anticommuting with the next generator
        constexpr int MAXI = kP3Items + 1;
        unsigned short osrc[MAXI];  // tile-local source: K index, or F index | 0x8000
        double val[MAXI];
        unsigned char cls[MAXI], nx[MAXI];
        unsigned cnt_k = 0, cnt_n = 0, cnt_r = 0;
        U128 l1{0ull, 0ull}, sq{0ull, 0ull};
        bool bad = false;
#pragma unroll
        for (int e = 0; e < MAXI; ++e) {
            cls[e] = 0;
            nx[e] = 0;
            val[e] = 0.0;
            osrc[e] = 0;
            if (lo_d + e >= hi_d) continue;
            bool take_k;
            if (ik >= nk) take_k = false;
            else if (jf >= nf) take_k = true;
            else take_k = key_le<W>(kkey(ik), fkey(jf));
            Key<W> key;
            double v;
            if (take_k) {
                key = kkey(ik);
                osrc[e] = (unsigned short)ik;
                const double vin = s_kv[ik];
                ++ik;
                bool anti, plus;
                branch_info(p, word_at<W>(key, p.i_word), word_at<W>(key, p.j_word), anti, plus);
                // commuting: the reference sums (v) + (+0), which is v for v != 0
                // and +0 for a zero (dropped below either way)
                v = anti ? __dmul_rn(vin, c) : vin;
                // the partner (if any) is the next merged element: sum it here
                if (jf < nf && key_eq<W>(fkey(jf), key)) v = __dadd_rn(v, s_fv[jf]);
            } else {
                key = fkey(jf);
                osrc[e] = (unsigned short)(0x8000u | (unsigned)jf);
                v = s_fv[jf];
                ++jf;
                // partner of the preceding cos child: already summed there
                if (ik > 0 && key_eq<W>(kkey(ik - 1), key)) continue;
            }
            if (!is_finite(v)) bad = true;
            if (is_zero(v)) continue;  // exact cancellation: dropped, no ledger entry
            val[e] = v;
            if (!key_is_zero<W>(key) && abs_bits(v) <= p.threshold_bits) {
                cls[e] = 2;
                ++cnt_r;
                if (!p.exact_ledger) {
                    U128 x1, x2;
                    fixed_terms(v, p.fx_unit1, p.fx_unit2, x1, x2);
                    u128_add(l1, x1);
                    u128_add(sq, x2);
                }
            } else {
                cls[e] = 1;
                ++cnt_k;
                if (p.has_next) {
                    const unsigned pi = site_symbol(word_at<W>(key, p.n_i_word), p.n_i_shift);
                    const unsigned pj = site_symbol(word_at<W>(key, p.n_j_word), p.n_j_shift);
                    if (anticommutes(p.n_qi, pi) != anticommutes(p.n_qj, pj)) {
                        const bool plus_n =
                            ((phase_exponent(p.n_qi, pi) + phase_exponent(p.n_qj, pj)) & 3u) == 1u;
                        nx[e] = plus_n ? 1 : 2;
                        ++cnt_n;
                    }
                }
            }
        }
        if (bad) atomicOr(&st->status, ST_NUMERIC);
        // block exclusive scans of the three counts in thread order
        unsigned sk_ = cnt_k, sn_ = cnt_n, sr_ = cnt_r;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const unsigned tk = __shfl_up_sync(0xffffffffu, sk_, off);
            const unsigned tn = __shfl_up_sync(0xffffffffu, sn_, off);
            const unsigned tr = __shfl_up_sync(0xffffffffu, sr_, off);
            if (lane >= (unsigned)off) {
                sk_ += tk;
                sn_ += tn;
                sr_ += tr;
            }
        }
        // ledger partials: exact 128-bit sums within the warp, then across warps
        U128 wl1 = l1, wsq = sq;
        if (!p.exact_ledger) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                u128_add(wl1, shfl_down_u128(wl1, off));
                u128_add(wsq, shfl_down_u128(wsq, off));
            }
        }
        if (lane == 31) {
            s_wk[warp] = sk_;
            s_wn[warp] = sn_;
            s_wr[warp] = sr_;
        }
        if (lane == 0) {
            s_l1[warp] = wl1;
            s_sq[warp] = wsq;
        }
        __syncthreads();
        unsigned wk_off = 0, wn_off = 0, wr_off = 0, tk_tot = 0, tn_tot = 0, tr_tot = 0;
        for (int w = 0; w < NW; ++w) {
            if (w < (int)warp) {
                wk_off += s_wk[w];
                wn_off += s_wn[w];
                wr_off += s_wr[w];
            }
            tk_tot += s_wk[w];
            tn_tot += s_wn[w];
            tr_tot += s_wr[w];
        }
        if (warp == 0) {
            const unsigned long long base =
                lookback_exclusive(b.p3_tiles, tile, pack2(tk_tot, tn_tot), &st->status,
                                   poll_limit(st, kLookbackPolls));
            if (lane == 0) {
                unsigned long long bk, bn;
                unpack2(base, bk, bn);
                s_base_k = bk;
                s_base_n = bn;
                if (!p.exact_ledger) {
                    U128 t1{0ull, 0ull}, t2{0ull, 0ull};
                    for (int w = 0; w < NW; ++w) {
                        u128_add(t1, s_l1[w]);
                        u128_add(t2, s_sq[w]);
                    }
                    b.partials[4 * tile] = t1.lo;
                    b.partials[4 * tile + 1] = t1.hi;
                    b.partials[4 * tile + 2] = t2.lo;
                    b.partials[4 * tile + 3] = t2.hi;
                }
                b.rem_count[tile] = tr_tot;
                if (tr_tot) atomicAdd(&st->removed, (unsigned long long)tr_tot);
                s_base_r = 0;
                if (tile == ntiles - 1) {
                    const unsigned long long n_out = bk + tk_tot, a_next = bn + tn_tot;
                    st->n_out = n_out;
                    st->a_next = a_next;
                    if (p.has_next && n_out + a_next > b.cap) atomicOr(&st->status, ST_CAPACITY);
                }
            }
        }
        if (p.exact_ledger && b.log && warp == 0) {
            // this tile's place among the rotation's removed values (key order)
            const unsigned long long rb = lookback_exclusive(b.p3r_tiles, tile, pack2(tr_tot, 0),
                                                             &st->status, poll_limit(st, kLookbackPolls));
            if (lane == 0) {
                unsigned long long r0, r1;
                unpack2(rb, r0, r1);
                s_base_r = __ldcg(&st->log_pos) + r0;
                if (s_base_r + tr_tot > b.log_cap) atomicOr(&st->status, ST_LOG);
            }
        }
        __syncthreads();
        unsigned long long ok = s_base_k + wk_off + (sk_ - cnt_k);
        unsigned long long on = s_base_n + wn_off + (sn_ - cnt_n);
        unsigned orr = wr_off + (sr_ - cnt_r);
        const double sn = p.n_s;
#pragma unroll
        for (int e = 0; e < MAXI; ++e) {
            if (cls[e] == 0) continue;
            if (cls[e] == 1) {
                const Key<W> key = (osrc[e] & 0x8000u) ? fkey(osrc[e] & 0x7fff) : kkey(osrc[e]);
                if (ok < b.cap) {
                    store_key<W>(b.out_keys, ok, key);
                    b.out_vals[ok] = val[e];
                } else {
                    atomicOr(&st->status, ST_CAPACITY);
                }
                ++ok;
                if (nx[e]) {
                    if (on < b.cap) {
                        const double y = __dmul_rn(val[e], sn);
                        store_key<W>(b.fk, on, key_xor<W>(key, MN));
                        reinterpret_cast<unsigned long long*>(b.fv)[on] =
                            dbits(y) ^ (nx[e] == 1 ? 0ull : kSignBit);
                    } else {
                        atomicOr(&st->status, ST_CAPACITY);
                    }
                    ++on;
                }
            } else {
                if (p.exact_ledger) {
                    if (!b.log) {
                        b.rem[tile * (unsigned long long)T + orr] = abs_of(val[e]);
                    } else if (s_base_r + orr < b.log_cap) {
                        b.log[s_base_r + orr] = abs_of(val[e]);
                    }
                }
                ++orr;
            }
        }
    }
    // the last CTA to finish commits the rotation
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(&st->merge_done, 1u) == (unsigned)(participants - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    commit_rotation<kP3Block>(p, b, ntiles);
}

// ------------------------------------------------ exact ledger after the call
// One thread per rotation: the reference's sequential removed-weight sums
// (engine/src/tpgp_rev.c:716-729 and upper_l2, :43-63, without MPFR) over the
// rotation's logged |v| in key order: l1 = upadd(l1, v), sq = upadd(sq,
// upmul(v, v)).  Values are loaded eight at a time ahead of the chain.
struct ChainSums {
    double l1, sq;
};
__global__ void __launch_bounds__(128) k_exact_chains(const double* log, const RotLog* rot_log,
                                                     const DeviceState* st, ChainSums* sums) {
    const unsigned long long done = __ldcg(&st->rotations_done);
    const unsigned long long r = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= done) return;
    const RotLog e = rot_log[r];
    double l1 = 0.0, sq = 0.0;
    if (e.counted) {
        unsigned long long k = 0;
        for (; k + 8 <= e.count; k += 8) {
            double v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) v[q] = __ldcg(log + e.off + k + q);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                l1 = up_add(l1, v[q]);
                sq = up_add(sq, up_mul(v[q], v[q]));
            }
        }
        for (; k < e.count; ++k) {
            const double v = __ldcg(log + e.off + k);
            l1 = up_add(l1, v);
            sq = up_add(sq, up_mul(v, v));
        }
    }
    sums[r] = ChainSums{l1, sq};
}

// One thread: the ledger update of commit_rotation (tpgp_rev.c:730-753) for
// the committed rotations in order, with its ENUMERIC and EBUDGET checks.
// The first rotation that fails decides the call's status, ahead of any
// failure a later rotation reported while the sums were deferred; the step
// is transactional, so the map is discarded as the reference discards it.
__global__ void k_exact_walk(const RotLog* rot_log, const ChainSums* sums, DeviceState* st,
                             double max_drop_l2) {
    const unsigned long long done = st->rotations_done;
    Ledger led = st->ledger;
    unsigned fail = 0;
    for (unsigned long long r = 0; r < done && !fail; ++r) {
        if (!rot_log[r].counted) continue;  // empty map: no ledger change
        const ChainSums x = sums[r];
        const double l2 = x.sq == 0.0 ? 0.0 : next_up(sqrt(x.sq));
        led.dropped_l1 = up_add(led.dropped_l1, x.l1);
        led.dropped_l2 = up_add(led.dropped_l2, l2);
        led.dropped_l2_squared = up_add(led.dropped_l2_squared, x.sq);
        led.arithmetic_l2 = up_add(led.arithmetic_l2, 0.0);
        if (!is_finite(led.dropped_l2) || !is_finite(led.arithmetic_l2)) fail = ST_NUMERIC;
        else if (max_drop_l2 != 0.0 && led.dropped_l2 > max_drop_l2) fail = ST_BUDGET;
    }
    const unsigned status = st->status;
    const unsigned infra = ST_CAPACITY | ST_LOG | ST_TIMEOUT | ST_ORDER;
    if (fail && !(status & infra)) {
        st->status = fail;
    } else if (!status) {
        st->ledger.dropped_l1 = led.dropped_l1;
        st->ledger.dropped_l2 = led.dropped_l2;
        st->ledger.dropped_l2_squared = led.dropped_l2_squared;
        st->ledger.arithmetic_l2 = led.arithmetic_l2;
    }
}

template <int W>
__global__ void __launch_bounds__(kP3Block, 3) k_merge(RotParams p, Buffers b) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    pdl_enter();
    phase_merge<W>(p, b, smem_raw, false, whole_grid());
}

// ============================================================== persistent
// One cooperative launch runs a whole list of rotations: the same phases as
// the per-kernel path, separated by grid barriers instead of kernel
// boundaries.  All CTAs are co-resident (cooperative launch), and every
// barrier wait is bounded: a wait that gives up sets ST_TIMEOUT and the CTA
// leaves the kernel, so no launch can spin forever.
constexpr unsigned kBarrierPolls = 1u << 24;

// false if the wait gave up
__device__ inline bool grid_barrier(DeviceState* st) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* gen = &st->bar_gen;
        const unsigned g = *gen;
        __threadfence();
        const unsigned arrived = atomicAdd(&st->bar_count, 1u);
        const unsigned limit = poll_limit(st, kBarrierPolls);
        int ok = 1;
        if (arrived == gridDim.x - 1 + st->bar_extra) {
            atomicExch(&st->bar_count, 0u);
            __threadfence();
            atomicAdd(&st->bar_gen, 1u);
        } else {
            unsigned polls = 0;
            while (*gen == g) {
                if (++polls > limit) {
                    atomicOr(&st->status, ST_TIMEOUT);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

struct StepArgs {
    const RotParams* ps;     // rotation list in device memory
    unsigned rotations;
    uint64_t* keys[3];       // the three map buffers
    double* vals[3];
    int x, y, z;             // step input, then the two ping-pong buffers
    Buffers scratch;         // fk..st, cap (in/out filled per rotation)
};

template <int W>
__global__ void __launch_bounds__(kP3Block, 2) k_step(StepArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    DeviceState* st = a.scratch.st;
    for (unsigned r = 0; r < a.rotations; ++r) {
        const RotParams& p = a.ps[r];
        const int in = r == 0 ? a.x : ((r - 1) % 2 == 0 ? a.y : a.z);
        const int out = r % 2 == 0 ? a.y : a.z;
        Buffers b = a.scratch;
        b.in_keys = a.keys[in];
        b.in_vals = a.vals[in];
        b.out_keys = a.keys[out];
        b.out_vals = a.vals[out];
        const Grid g = whole_grid();
        if (r == 0) {
            phase_classify<W>(p, b, g);
            if (!grid_barrier(st)) return;
        }
        // phases skip their work once the status is set; the merge phase
        // still elects a committing CTA, which raises st->stop
        if (p.nth <= 4) phase_flip<W, 4>(p, b, smem_raw, g);
        else phase_flip<W, 6>(p, b, smem_raw, g);
        if (!grid_barrier(st)) return;
        phase_partition<W>(p, b, g);
        if (!grid_barrier(st)) return;
        phase_merge<W>(p, b, smem_raw, true, g);
        if (!grid_barrier(st)) return;
        // written only by the committing CTA before this barrier: uniform
        if (*reinterpret_cast<volatile unsigned*>(&st->stop)) return;
    }
}

// ================================================================= batched
// Many independent maps ("items": powder orientations, disorder realizations,
// served requests) advanced by one launch: each item is owned by one
// thread-block cluster of G CTAs (G = 1, 2, 4 or 8, chosen by the autotuner),
// which runs the item's whole rotation list with the same phases as above.
// Phases are separated by the hardware cluster barrier (release/acquire at
// cluster scope; a cluster of one CTA is a plain CTA barrier), so no software
// spin-wait is involved.  Items finish independently; the hardware scheduler
// starts the next clusters as SMs free up.
struct BatchItem {
    const RotParams* ps;   // this item's rotation list (device memory)
    unsigned rotations;
    unsigned active;       // 0: skip (finished or failed item)
    uint64_t* keys[3];
    double* vals[3];
    int x, y, z;
    int final_buf;         // buffer holding the map after the rotations
    unsigned n_spins;
    unsigned table_slots;  // > 0: the step runs in a CTA-local hash table of this size
    Buffers scratch;       // the item's own fk..st, cap
};

__device__ __forceinline__ void cluster_barrier() {
    __threadfence();
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;"
                 ::: "memory");
}
__device__ __forceinline__ unsigned cluster_rank() {
    unsigned r;
    asm("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cluster_size() {
    unsigned n;
    asm("mov.u32 %0, %%cluster_nctarank;" : "=r"(n));
    return n;
}

template <int W>
__global__ void __launch_bounds__(kP3Block, 2) k_batch(const BatchItem* items, const unsigned* ids) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Grid g{cluster_rank(), cluster_size()};
    const BatchItem& it = items[ids[blockIdx.x / g.ncta]];
    if (!it.active) return;  // uniform across the cluster
    DeviceState* st = it.scratch.st;
    for (unsigned r = 0; r < it.rotations; ++r) {
        const RotParams& p = it.ps[r];
        const int in = r == 0 ? it.x : ((r - 1) % 2 == 0 ? it.y : it.z);
        const int out = r % 2 == 0 ? it.y : it.z;
        Buffers b = it.scratch;
        b.in_keys = it.keys[in];
        b.in_vals = it.vals[in];
        b.out_keys = it.keys[out];
        b.out_vals = it.vals[out];
        if (r == 0) {
            phase_classify<W>(p, b, g);
            cluster_barrier();
        }
        if (p.nth <= 4) phase_flip<W, 4>(p, b, smem_raw, g);
        else phase_flip<W, 6>(p, b, smem_raw, g);
        cluster_barrier();
        phase_partition<W>(p, b, g);
        cluster_barrier();
        phase_merge<W>(p, b, smem_raw, true, g);
        cluster_barrier();
        if (__ldcg(&st->stop)) break;  // written by the committing CTA before the barrier
    }
}

// Per item, the coefficient of each weight-one key `pauli` at site s after a
// batched step (0 if absent): out[item * 128 + s].  One CTA per item.
template <int W>
__global__ void k_batch_readout(const BatchItem* items, const unsigned* ids, unsigned pauli,
                                double* out) {
    const unsigned item = ids[blockIdx.x];
    const BatchItem& it = items[item];
    const unsigned s = threadIdx.x;
    double v = 0.0;
    if (it.active && s < it.n_spins) {
        const uint64_t* keys = it.keys[it.final_buf];
        const double* vals = it.vals[it.final_buf];
        const unsigned long long len = __ldcg(&it.scratch.st->n);
        Key<W> target;
#pragma unroll
        for (int w = 0; w < W; ++w) target.w[w] = 0;
#pragma unroll
        for (int w = 0; w < W; ++w)
            if (w == (int)(s / 32)) target.w[w] = (uint64_t)pauli << (2 * (s % 32));
        unsigned long long lo = 0, hi = len;
        while (lo < hi) {
            const unsigned long long mid = lo + (hi - lo) / 2;
            if (key_less<W>(load_key<W>(keys, mid), target)) lo = mid + 1;
            else hi = mid;
        }
        if (lo < len && key_eq<W>(load_key<W>(keys, lo), target)) v = __ldcg(vals + lo);
    }
    if (s < 128) out[(size_t)item * 128 + s] = v;
}

}  // namespace tg
