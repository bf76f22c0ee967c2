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
//                 look-back compaction of kept terms (and of removed ones for
//                 the exact ledger), per-tile ledger partial sums     [P3b]
//   k_commit    : ledger update, cap and budget checks, state for the next
//                 rotation                                            [commit]
#pragma once
#include "common.cuh"

namespace tg {

// ------------------------------------------------------------- parameters
struct RotParams {
    int i_word, i_shift, j_word, j_shift;  // word and bit offset of sites i, j
    unsigned qi, qj;
    double c, s;            // host-computed cos/sin (never evaluated on device)
    double threshold;
    uint64_t mask[4];       // Q's bits: qi at site i, qj at site j
    int nlev;               // number of mask bits (radix digits), 0..4
    int mbit[4];            // mask bit positions, descending
    int nth;                // distinct digit-boundary thresholds
    int th[8];              // threshold bit positions
    int lev_lo[4], lev_hi[4];  // index in th of mbit[l] and mbit[l] + 1
    int exact_ledger;       // 1: removed values kept in order for a sequential ledger
    unsigned long long max_terms;
    double max_drop_l2;
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
    double* rem;                   // removed |v| in key order (exact ledger)
    unsigned long long* splits;    // merge-path split (i, j) per tile boundary
    double* partials;              // per-tile (l1, sq) partial ledger sums
    unsigned long long* p1_tiles;  // look-back words
    unsigned long long* p3_tiles;
    DeviceState* st;
    unsigned long long cap;        // terms each map / child buffer holds
};

constexpr int kP1Block = 256, kP1Items = 8, kP1Tile = kP1Block * kP1Items;
constexpr int kP2Block = 256, kP2Items = 8, kP2Tile = kP2Block * kP2Items;
constexpr int kP3Block = 256, kP3Items = 8, kP3Tile = kP3Block * kP3Items;
constexpr int kCommitBlock = 1024;
constexpr int kBlInf = 0x7fff;  // digit-boundary level of element 0
static_assert(kP1Items * (kP1Block / 32) == 64, "P1 row/warp scan assumes 64 entries");

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

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
__global__ void __launch_bounds__(kP1Block) k_classify(RotParams p, Buffers b) {
    constexpr int NW = kP1Block / 32;
    __shared__ unsigned s_counts[kP1Items * NW];
    __shared__ unsigned long long s_tile, s_base;
    DeviceState* st = b.st;
    if (st->status) return;
    const unsigned long long n = st->n;
    const unsigned long long ntiles = (n + kP1Tile - 1) / kP1Tile;
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
                const uint64_t wi = __ldg(b.in_keys + k * W + p.i_word);
                const uint64_t wj = __ldg(b.in_keys + k * W + p.j_word);
                branch_info(p, wi, wj, anti[e], plus[e]);
                const double v = __ldg(b.in_vals + k);
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
                lookback_exclusive(b.p1_tiles, tile, pack2(total, 0), &st->status);
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
            const double v = __ldg(b.in_vals + k);
            const double y = __dmul_rn(v, p.s);
            store_key<W>(b.fk, x, key_xor<W>(key, M));
            b.fv[x] = plus[e] ? y : -y;
        }
    }
}

// ======================================================================= P2
// Galloping search over the anticommuting sequence A (A[y] = fk[y] xor M) for
// the start of the run of elements that share all bits >= theta with A[from]
// (backward = true), or for the first element after that run (forward).
template <int W>
__device__ unsigned long long run_edge(const uint64_t* fk, const Key<W>& M,
                                       unsigned long long a, unsigned long long from,
                                       int theta, bool backward) {
    const Key<W> target = key_high<W>(key_xor<W>(load_key_coherent<W>(fk, from), M), theta);
    auto same = [&](unsigned long long y) {
        return key_eq<W>(key_high<W>(key_xor<W>(load_key_coherent<W>(fk, y), M), theta), target);
    };
    if (backward) {
        // find the smallest y <= from with same(y); same(from) holds
        unsigned long long good = from, step = 1;
        unsigned long long bad_pos = ~0ull;  // ~0 = "before 0"
        while (true) {
            if (good < step) {
                if (same(0)) return 0;
                bad_pos = 0;
                break;
            }
            const unsigned long long y = good - step;
            if (same(y)) {
                good = y;
                step <<= 1;
            } else {
                bad_pos = y;
                break;
            }
        }
        // invariant: !same(bad_pos), same(good), bad_pos < good
        while (good - bad_pos > 1) {
            const unsigned long long mid = bad_pos + (good - bad_pos) / 2;
            if (same(mid)) good = mid;
            else bad_pos = mid;
        }
        return good;
    } else {
        // find the smallest y > from with !same(y), or a
        unsigned long long good = from, step = 1, bad_pos = a;
        while (true) {
            const unsigned long long y = good + step;
            if (y >= a) break;
            if (same(y)) {
                good = y;
                step <<= 1;
            } else {
                bad_pos = y;
                break;
            }
        }
        while (bad_pos - good > 1) {
            const unsigned long long mid = good + (bad_pos - good) / 2;
            if (same(mid)) good = mid;
            else bad_pos = mid;
        }
        return bad_pos;
    }
}

template <int W>
__global__ void __launch_bounds__(kP2Block) k_flip_sort(RotParams p, Buffers b) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint64_t* s_keys = reinterpret_cast<uint64_t*>(smem_raw);                 // [tile][W]
    double* s_vals = reinterpret_cast<double*>(s_keys + (size_t)kP2Tile * W);  // [tile]
    short* s_bl = reinterpret_cast<short*>(s_vals + kP2Tile);                 // [tile]
    __shared__ long long s_gprev[8], s_gnext[8];
    __shared__ long long s_wprev[kP2Block / 32][8], s_wnext[kP2Block / 32][8];

    DeviceState* st = b.st;
    if (st->status) return;
    const unsigned long long a = st->a;
    if (a == 0 || p.nlev == 0) return;
    const unsigned long long ntiles = (a + kP2Tile - 1) / kP2Tile;
    const Key<W> M = mask_key<W>(p);
    const int nth = p.nth;
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;

    for (unsigned long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const unsigned long long x0 = tile * kP2Tile;
        const int len = (int)((a - x0) < (unsigned long long)kP2Tile ? (a - x0) : (unsigned long long)kP2Tile);
        const unsigned long long x1 = x0 + len;
        __syncthreads();
        for (int e = threadIdx.x; e < len; e += kP2Block) {
            const Key<W> k = load_key<W>(b.fk, x0 + e);
#pragma unroll
            for (int w = 0; w < W; ++w) s_keys[(size_t)e * W + w] = k.w[w];
            s_vals[e] = __ldg(b.fv + x0 + e);
        }
        // run edges outside the tile for every threshold (galloping searches)
        if (threadIdx.x < 2 * nth) {
            const int q = threadIdx.x % nth;
            if (threadIdx.x < nth) {
                // last y < x0 with bl(y) >= th[q]: start of the run holding x0-1
                s_gprev[q] = x0 == 0 ? -1 : (long long)run_edge<W>(b.fk, M, a, x0 - 1, p.th[q], true);
            } else {
                // first y >= x1 with bl(y) >= th[q] (a if none)
                s_gnext[q] = x1 >= a ? (long long)a
                                     : (long long)max(x1, run_edge<W>(b.fk, M, a, x1 - 1, p.th[q], false));
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
        long long lprev[8], lnext[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            lprev[q] = -1;
            lnext[q] = LLONG_MAX;
        }
        for (int e = 0; e < kP2Items; ++e) {
            const int te = e0 + e;
            if (te >= len) break;
            const int bl = s_bl[te];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                if (q < nth && bl >= p.th[q]) {
                    lprev[q] = (long long)(x0 + te);
                    if (lnext[q] == LLONG_MAX) lnext[q] = (long long)(x0 + te);
                }
            }
        }
        // exclusive cross-thread scans: max of earlier threads' last, min of later threads' first
        long long cprev[8], cnext[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            long long incl = lprev[q];
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const long long t = __shfl_up_sync(0xffffffffu, incl, off);
                if (lane >= (unsigned)off) incl = max(incl, t);
            }
            long long excl = __shfl_up_sync(0xffffffffu, incl, 1);
            if (lane == 0) excl = -1;
            cprev[q] = excl;
            if (lane == 31) s_wprev[warp][q] = incl;
            long long rincl = lnext[q];
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const long long t = __shfl_down_sync(0xffffffffu, rincl, off);
                if (lane + off < 32) rincl = min(rincl, t);
            }
            long long rexcl = __shfl_down_sync(0xffffffffu, rincl, 1);
            if (lane == 31) rexcl = LLONG_MAX;
            cnext[q] = rexcl;
            if (lane == 0) s_wnext[warp][q] = rincl;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            if (q >= nth) break;
            long long pv = -1, nv = LLONG_MAX;
            for (int w = 0; w < (int)warp; ++w) pv = max(pv, s_wprev[w][q]);
            for (int w = (int)warp + 1; w < kP2Block / 32; ++w) nv = min(nv, s_wnext[w][q]);
            cprev[q] = max(cprev[q], pv);
            cnext[q] = min(cnext[q], nv);
            if (cprev[q] < 0) cprev[q] = s_gprev[q];
            if (cnext[q] == LLONG_MAX) cnext[q] = s_gnext[q];
        }
        // forward pass: displacement of the digits that are 1 (move back by n0)
        long long disp[kP2Items];
        {
            long long run[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) run[q] = cprev[q];
            for (int e = 0; e < kP2Items; ++e) {
                const int te = e0 + e;
                disp[e] = 0;
                if (te >= len) continue;
                const int bl = s_bl[te];
                const long long x = (long long)(x0 + te);
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    if (q < nth && bl >= p.th[q]) run[q] = x;
                Key<W> fkey;
#pragma unroll
                for (int w = 0; w < W; ++w) fkey.w[w] = s_keys[(size_t)te * W + w];
#pragma unroll
                for (int l = 0; l < 4; ++l) {
                    if (l >= p.nlev) break;
                    // digit of the unflipped key = flipped bit xor 1
                    if (key_bit<W>(fkey, p.mbit[l]) == 0) {  // original digit 1
                        const long long sp = pick<8>(run, p.lev_lo[l]), sg = pick<8>(run, p.lev_hi[l]);
                        disp[e] -= (sp == sg) ? 0 : (sp - sg);
                    }
                }
            }
        }
        // backward pass: displacement of the digits that are 0 (move ahead by n1)
        {
            long long run[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) run[q] = cnext[q];
            for (int e = kP2Items - 1; e >= 0; --e) {
                const int te = e0 + e;
                if (te >= len) continue;
                const int bl = s_bl[te];
                const long long x = (long long)(x0 + te);
                Key<W> fkey;
#pragma unroll
                for (int w = 0; w < W; ++w) fkey.w[w] = s_keys[(size_t)te * W + w];
#pragma unroll
                for (int l = 0; l < 4; ++l) {
                    if (l >= p.nlev) break;
                    if (key_bit<W>(fkey, p.mbit[l]) == 1) {  // original digit 0
                        const long long sp = pick<8>(run, p.lev_lo[l]), en = pick<8>(run, p.lev_hi[l]);
                        disp[e] += (sp == en) ? 0 : (en - sp);
                    }
                }
                const unsigned long long dest = (unsigned long long)(x + disp[e]);
                if (dest < a) {
                    store_key<W>(b.sk, dest, fkey);
                    b.sv[dest] = s_vals[te];
                } else {
                    atomicOr(&st->status, ST_ORDER);
                }
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    if (q < nth && bl >= p.th[q]) run[q] = x;
            }
        }
    }
}

// ====================================================================== P3a
template <int W>
__global__ void k_partition(RotParams p, Buffers b) {
    DeviceState* st = b.st;
    if (st->status) return;
    const unsigned long long n = st->n, a = st->a, L = n + a;
    const unsigned long long ntiles = (L + kP3Tile - 1) / kP3Tile;
    for (unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
         t <= ntiles; t += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long d = min(t * (unsigned long long)kP3Tile, L);
        unsigned long long lo = d > a ? d - a : 0, hi = min(d, n);
        while (lo < hi) {
            const unsigned long long mid = lo + (hi - lo) / 2;
            // is K[mid] merged before S[d - mid - 1]?  (ties: cos list first)
            if (key_le<W>(load_key<W>(b.in_keys, mid), load_key<W>(b.sk, d - mid - 1)))
                lo = mid + 1;
            else
                hi = mid;
        }
        unsigned long long i = lo, j = d - lo;
        // keep a (cos, sin) pair with equal keys inside one tile
        if (i > 0 && j < a && key_eq<W>(load_key<W>(b.in_keys, i - 1), load_key<W>(b.sk, j))) ++j;
        b.splits[2 * t] = i;
        b.splits[2 * t + 1] = j;
    }
}

// ====================================================================== P3b
template <int W>
__global__ void __launch_bounds__(kP3Block) k_merge(RotParams p, Buffers b) {
    constexpr int T = kP3Tile + 1;  // one extra slot for a pair moved across the boundary
    constexpr int NW = kP3Block / 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint64_t* s_kk = reinterpret_cast<uint64_t*>(smem_raw);       // cos-list keys [T][W]
    uint64_t* s_fk = s_kk + (size_t)T * W;                        // sorted flipped keys
    double* s_kv = reinterpret_cast<double*>(s_fk + (size_t)T * W);
    double* s_fv = s_kv + T;
    unsigned* s_src = reinterpret_cast<unsigned*>(s_fv + T);      // merged order
    __shared__ unsigned long long s_tile, s_base_k, s_base_r;
    __shared__ unsigned s_wk[NW], s_wr[NW];
    __shared__ double s_l1[NW], s_sq[NW];

    DeviceState* st = b.st;
    if (st->status) return;
    const unsigned long long n = st->n, a = st->a, L = n + a;
    const unsigned long long ntiles = (L + kP3Tile - 1) / kP3Tile;
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    const double c = p.c;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_tile = atomicAdd(&st->p3_counter, 1u);
        __syncthreads();
        const unsigned long long tile = s_tile;
        if (tile >= ntiles) break;
        const unsigned long long i0 = b.splits[2 * tile], j0 = b.splits[2 * tile + 1];
        const unsigned long long i1 = b.splits[2 * tile + 2], j1 = b.splits[2 * tile + 3];
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
            s_kv[e] = __ldg(b.in_vals + i0 + e);
        }
        for (int e = threadIdx.x; e < nf; e += kP3Block) {
            const Key<W> k = load_key<W>(b.sk, j0 + e);
#pragma unroll
            for (int w = 0; w < W; ++w) s_fk[(size_t)e * W + w] = k.w[w];
            s_fv[e] = b.sv[j0 + e];
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
        // each thread merges its own output range [lo, hi)
        const int lo_d = min(len, (int)threadIdx.x * kP3Items);
        const int hi_d = threadIdx.x == kP3Block - 1 ? len : min(len, lo_d + kP3Items);
        {
            int lo = max(0, lo_d - nf), hi = min(lo_d, nk);
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (key_le<W>(kkey(mid), fkey(lo_d - mid - 1))) lo = mid + 1;
                else hi = mid;
            }
            int ik = lo, jf = lo_d - lo;
            for (int d = lo_d; d < hi_d; ++d) {
                bool take_k;
                if (ik >= nk) take_k = false;
                else if (jf >= nf) take_k = true;
                else take_k = key_le<W>(kkey(ik), fkey(jf));
                s_src[d] = take_k ? (unsigned)ik++ : (0x80000000u | (unsigned)jf++);
            }
        }
        __syncthreads();
        // classify: 0 drop, 1 keep, 2 removed
        constexpr int MAXI = kP3Items + 1;
        double val[MAXI];
        unsigned char cls[MAXI];
        unsigned cnt_k = 0, cnt_r = 0;
        double l1 = 0.0, sq = 0.0;
        bool bad = false;
#pragma unroll
        for (int e = 0; e < MAXI; ++e) {
            const int d = lo_d + e;
            cls[e] = 0;
            val[e] = 0.0;
            if (d >= hi_d) continue;
            const unsigned s = s_src[d];
            Key<W> key;
            double v;
            if (s & 0x80000000u) {
                const int f = (int)(s & 0x7fffffffu);
                key = fkey(f);
                if (d > 0) {
                    const unsigned sp = s_src[d - 1];
                    // partner of the preceding cos child: already summed there
                    if (!(sp & 0x80000000u) && key_eq<W>(kkey((int)sp), key)) continue;
                }
                v = s_fv[f];
            } else {
                const int k = (int)s;
                key = kkey(k);
                const double vin = s_kv[k];
                bool anti, plus;
                branch_info(p, word_at<W>(key, p.i_word), word_at<W>(key, p.j_word), anti, plus);
                v = anti ? __dmul_rn(vin, c) : __dadd_rn(vin, 0.0);
                if (d + 1 < len) {
                    const unsigned sn = s_src[d + 1];
                    if ((sn & 0x80000000u) && key_eq<W>(fkey((int)(sn & 0x7fffffffu)), key))
                        v = __dadd_rn(v, s_fv[sn & 0x7fffffffu]);
                }
            }
            if (!is_finite(v)) bad = true;
            if (v == 0.0) continue;  // exact cancellation: dropped, no ledger entry
            val[e] = v;
            if (!key_is_zero<W>(key) && fabs(v) <= p.threshold) {
                cls[e] = 2;
                ++cnt_r;
                const double av = fabs(v);
                l1 = up_add(l1, av);
                sq = up_add(sq, up_mul(v, v));
            } else {
                cls[e] = 1;
                ++cnt_k;
            }
        }
        if (bad) atomicOr(&st->status, ST_NUMERIC);
        // block exclusive scan of (kept, removed) counts in thread order
        unsigned ik = cnt_k, ir = cnt_r;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const unsigned tk = __shfl_up_sync(0xffffffffu, ik, off);
            const unsigned tr = __shfl_up_sync(0xffffffffu, ir, off);
            if (lane >= (unsigned)off) {
                ik += tk;
                ir += tr;
            }
        }
        // ledger partials: deterministic tree within the warp, then across warps
        double wl1 = l1, wsq = sq;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const double o1 = __shfl_down_sync(0xffffffffu, wl1, off);
            const double o2 = __shfl_down_sync(0xffffffffu, wsq, off);
            wl1 = up_add(wl1, o1);
            wsq = up_add(wsq, o2);
        }
        if (lane == 31) {
            s_wk[warp] = ik;
            s_wr[warp] = ir;
        }
        if (lane == 0) {
            s_l1[warp] = wl1;
            s_sq[warp] = wsq;
        }
        __syncthreads();
        unsigned wk_off = 0, wr_off = 0, tk_tot = 0, tr_tot = 0;
        for (int w = 0; w < NW; ++w) {
            if (w < (int)warp) {
                wk_off += s_wk[w];
                wr_off += s_wr[w];
            }
            tk_tot += s_wk[w];
            tr_tot += s_wr[w];
        }
        if (warp == 0) {
            const unsigned long long base =
                lookback_exclusive(b.p3_tiles, tile, pack2(tk_tot, tr_tot), &st->status);
            if (lane == 0) {
                unsigned long long bk, br;
                unpack2(base, bk, br);
                s_base_k = bk;
                s_base_r = br;
                double t1 = 0.0, t2 = 0.0;
                for (int w = 0; w < NW; ++w) {
                    t1 = up_add(t1, s_l1[w]);
                    t2 = up_add(t2, s_sq[w]);
                }
                b.partials[2 * tile] = t1;
                b.partials[2 * tile + 1] = t2;
                if (tile == ntiles - 1) {
                    st->n_out = bk + tk_tot;
                    st->removed = br + tr_tot;
                    st->p3_tiles = ntiles;
                }
            }
        }
        __syncthreads();
        unsigned long long ok = s_base_k + wk_off + (ik - cnt_k);
        unsigned long long orr = s_base_r + wr_off + (ir - cnt_r);
#pragma unroll
        for (int e = 0; e < MAXI; ++e) {
            if (cls[e] == 0) continue;
            const int d = lo_d + e;
            const unsigned s = s_src[d];
            if (cls[e] == 1) {
                if (ok < b.cap) {
                    const Key<W> key = (s & 0x80000000u) ? fkey((int)(s & 0x7fffffffu)) : kkey((int)s);
                    store_key<W>(b.out_keys, ok, key);
                    b.out_vals[ok] = val[e];
                } else {
                    atomicOr(&st->status, ST_CAPACITY);
                }
                ++ok;
            } else {
                if (p.exact_ledger && orr < b.cap) b.rem[orr] = fabs(val[e]);
                ++orr;
            }
        }
    }
}

// =================================================================== commit
// Ledger update of tpgp_rev.c:730-753 (non-validated), then reset of the
// per-rotation device state.  One block.
__global__ void __launch_bounds__(kCommitBlock) k_commit(RotParams p, Buffers b) {
    __shared__ double s_l1[kCommitBlock / 32], s_sq[kCommitBlock / 32];
    __shared__ unsigned long long s_n, s_a, s_t1, s_t3;
    DeviceState* st = b.st;
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        s_n = st->n;
        s_a = st->a;
        // clamp to the look-back arrays (n + a can exceed cap when the
        // rotation ran out of room)
        const unsigned long long t1_max = (b.cap + kP1Tile - 1) / kP1Tile;
        const unsigned long long t3_max = (b.cap + kP3Tile - 1) / kP3Tile;
        s_t1 = min((s_n + kP1Tile - 1) / kP1Tile, t1_max);
        s_t3 = min((s_n + s_a + kP3Tile - 1) / kP3Tile, t3_max);
    }
    __syncthreads();
    const unsigned status = st->status;
    const unsigned long long n = s_n;
    double l1 = 0.0, sq = 0.0;
    if (!status && n > 0) {
        const unsigned long long removed = st->removed;
        if (p.exact_ledger) {
            // the reference's sequential order: sorted key order, one thread
            if (threadIdx.x == 0) {
                for (unsigned long long k = 0; k < removed; ++k) {
                    const double v = b.rem[k];
                    l1 = up_add(l1, v);
                    sq = up_add(sq, up_mul(v, v));
                }
            }
        } else {
            // deterministic tree over the per-tile partials (fixed shape)
            const unsigned long long nt = st->p3_tiles;
            const unsigned long long per = (nt + kCommitBlock - 1) / kCommitBlock;
            const unsigned long long lo = threadIdx.x * per, hi = min(nt, lo + per);
            for (unsigned long long t = lo; t < hi; ++t) {
                l1 = up_add(l1, b.partials[2 * t]);
                sq = up_add(sq, b.partials[2 * t + 1]);
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const double o1 = __shfl_down_sync(0xffffffffu, l1, off);
                const double o2 = __shfl_down_sync(0xffffffffu, sq, off);
                l1 = up_add(l1, o1);
                sq = up_add(sq, o2);
            }
            if (lane == 0) {
                s_l1[warp] = l1;
                s_sq[warp] = sq;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                l1 = 0.0;
                sq = 0.0;
                for (int w = 0; w < kCommitBlock / 32; ++w) {
                    l1 = up_add(l1, s_l1[w]);
                    sq = up_add(sq, s_sq[w]);
                }
            }
        }
        if (threadIdx.x == 0) {
            const unsigned long long n_out = st->n_out;
            unsigned fail = 0;
            if (p.max_terms && n_out > p.max_terms) fail = ST_CAP;
            Ledger next = st->ledger;
            if (!fail) {
                const double l2 = sq == 0.0 ? 0.0 : next_up(sqrt(sq));
                next.dropped_l1 = up_add(next.dropped_l1, l1);
                next.dropped_l2 = up_add(next.dropped_l2, l2);
                next.dropped_l2_squared = up_add(next.dropped_l2_squared, sq);
                next.arithmetic_l2 = up_add(next.arithmetic_l2, 0.0);
                next.rotations += 1;
                if (removed) next.removal_events += 1;
                if (n_out > next.peak_terms) next.peak_terms = n_out;
                next.arithmetic_enclosed = 0;
                if (!is_finite(next.dropped_l2) || !is_finite(next.arithmetic_l2)) fail = ST_NUMERIC;
                else if (p.max_drop_l2 != 0.0 && next.dropped_l2 > p.max_drop_l2) fail = ST_BUDGET;
            }
            if (fail) {
                atomicOr(&st->status, fail);
            } else {
                st->ledger = next;
                st->n = n_out;
                st->rotations_done += 1;
                st->terms_in += n;
            }
        }
    } else if (!status && threadIdx.x == 0) {
        st->rotations_done += 1;  // empty map: a no-op rotation, no ledger change
    }
    __syncthreads();
    // reset per-rotation scratch: look-back words and tile counters
    for (unsigned long long t = threadIdx.x; t < s_t1 + 1; t += kCommitBlock) b.p1_tiles[t] = 0;
    for (unsigned long long t = threadIdx.x; t < s_t3 + 1; t += kCommitBlock) b.p3_tiles[t] = 0;
    if (threadIdx.x == 0) {
        st->p1_counter = 0;
        st->p3_counter = 0;
        st->a = 0;
        st->n_out = 0;
        st->removed = 0;
    }
}

}  // namespace tg
