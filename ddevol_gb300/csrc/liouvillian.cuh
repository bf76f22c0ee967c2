// The exact algebraic generator -i[H, A] of a device-resident map, in
// binary64 with no pruning, bitwise the reference's tpgp_liouvillian
// (engine/src/tpgp_rev.c:810-857).
//
// The reference adds, for each term in array order and each input key in key
// order, the contribution (2h) * v * (+1 if the phase exponent is 1, else -1)
// of every anticommuting key into its output key K xor Q (tpgp_map_add:
// running RN sums, a zero sum removes the key, a nonfinite contribution or
// sum is ENUMERIC).  A key's value is therefore the sequential RN sum of its
// contributions in (term, input key) order, kept when nonzero; later
// contributions after a cancellation to zero start from that zero, which
// gives the same sums.  Here:
//   1. k_lv_count: per (term, tile of 1024 keys) the anticommuting keys;
//   2. the host scans those counts in (term, tile) order;
//   3. k_lv_emit: every contribution written at its (term, key) rank, so the
//      buffer is in the reference's addition order;
//   4. a stable onesweep sort by key keeps that order among equal keys;
//   5. k_lv_sum: one thread per run of equal keys adds the run sequentially;
//   6. k_lv_kept / k_lv_write: the nonzero sums, compacted in key order.
#pragma once
#include "onesweep.cuh"

namespace tg {

constexpr int kLvBlock = 256, kLvItems = 4, kLvTile = kLvBlock * kLvItems;

// One term of the generator.  anti / plus: bit 4 pi + pj set when a key with
// symbols (pi, pj) at the term's sites anticommutes with it / has phase
// exponent 1 (tpgp_rev.c:414-417); h2 = 2h (exact).
struct LvTerm {
    int i_word, i_shift, j_word, j_shift;
    unsigned anti, plus;
    uint64_t mask[4];
    double h2;
};

template <int W>
__device__ __forceinline__ unsigned lv_index(const LvTerm& t, const Key<W>& k) {
    const unsigned pi = site_symbol(word_at<W>(k, t.i_word), t.i_shift);
    const unsigned pj = site_symbol(word_at<W>(k, t.j_word), t.j_shift);
    return 4u * pi + pj;
}

// counts[t * tiles + tile]: anticommuting keys of the tile for term t.
template <int W>
__global__ void __launch_bounds__(kLvBlock) k_lv_count(const uint64_t* keys, unsigned long long n,
                                                      const LvTerm* terms, unsigned t0,
                                                      unsigned* counts, unsigned long long tiles) {
    __shared__ unsigned s_n;
    const LvTerm& t = terms[t0 + blockIdx.y];
    if (threadIdx.x == 0) s_n = 0u;
    __syncthreads();
    unsigned mine = 0;
    const unsigned long long base = (unsigned long long)blockIdx.x * kLvTile;
#pragma unroll
    for (int e = 0; e < kLvItems; ++e) {
        const unsigned long long k = base + (unsigned long long)e * kLvBlock + threadIdx.x;
        if (k < n) mine += (t.anti >> lv_index<W>(t, load_key<W>(keys, k))) & 1u;
    }
    mine = __reduce_add_sync(0xffffffffu, mine);
    if ((threadIdx.x & 31u) == 0 && mine) atomicAdd(&s_n, mine);
    __syncthreads();
    if (threadIdx.x == 0) counts[(size_t)(t0 + blockIdx.y) * tiles + blockIdx.x] = s_n;
}

// Writes every contribution at offsets[t * tiles + tile] + its rank in key
// order within the tile.
template <int W>
__global__ void __launch_bounds__(kLvBlock) k_lv_emit(const uint64_t* keys, const double* vals,
                                                     unsigned long long n, const LvTerm* terms,
                                                     unsigned t0, const unsigned long long* offsets,
                                                     unsigned long long tiles, uint64_t* out_keys,
                                                     unsigned long long* out_vals, unsigned* status) {
    __shared__ unsigned s_warp[kLvItems][kLvBlock / 32];
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const LvTerm& t = terms[t0 + blockIdx.y];
    const unsigned long long base = (unsigned long long)blockIdx.x * kLvTile;
    Key<W> key[kLvItems];
    unsigned long long bits[kLvItems];
    bool on[kLvItems];
    unsigned rank[kLvItems];
    bool bad = false;
#pragma unroll
    for (int e = 0; e < kLvItems; ++e) {
        const unsigned long long k = base + (unsigned long long)e * kLvBlock + tid;
        on[e] = false;
        bits[e] = 0ull;
        if (k < n) {
            key[e] = load_key<W>(keys, k);
            const unsigned idx = lv_index<W>(t, key[e]);
            on[e] = (t.anti >> idx) & 1u;
            if (on[e]) {
                // (2h) * v, then the sign of the phase (tpgp_rev.c:831)
                double v = __dmul_rn(t.h2, __ldcg(vals + k));
                if (!((t.plus >> idx) & 1u)) v = negate(v);
                if (!is_finite(v)) bad = true;
                bits[e] = dbits(v);
#pragma unroll
                for (int w = 0; w < W; ++w) key[e].w[w] ^= t.mask[w];
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, on[e]);
        rank[e] = __popc(m & lanemask_lt());
        if (lane == 0) s_warp[e][warp] = __popc(m);
    }
    if (bad) atomicOr(status, ST_NUMERIC);
    __syncthreads();
    const unsigned long long off = offsets[(size_t)(t0 + blockIdx.y) * tiles + blockIdx.x];
    unsigned before = 0;  // contributions of earlier rounds and of earlier warps in this round
#pragma unroll
    for (int e = 0; e < kLvItems; ++e) {
        unsigned in_round = 0;
        for (unsigned w = 0; w < kLvBlock / 32; ++w) {
            if (w < warp) in_round += s_warp[e][w];
        }
        if (on[e]) {
            const unsigned long long at = off + before + in_round + rank[e];
            store_key<W>(out_keys, at, key[e]);
            out_vals[at] = bits[e];
        }
        for (unsigned w = 0; w < kLvBlock / 32; ++w) before += s_warp[e][w];
    }
}

// Sum of each run of equal keys (sorted), in buffer order, at the run's
// first index; zero elsewhere and for a run that sums to zero.
template <int W>
__global__ void __launch_bounds__(256) k_lv_sum(const uint64_t* keys, const unsigned long long* vals,
                                               const unsigned long long* count,
                                               unsigned long long* sums, unsigned* status) {
    const unsigned long long n = *count;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    bool bad = false;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += stride) {
        const Key<W> k = load_key<W>(keys, i);
        unsigned long long out = 0ull;
        if (i == 0 || !key_eq<W>(load_key<W>(keys, i - 1), k)) {
            double s = from_bits(__ldcg(vals + i));
            for (unsigned long long j = i + 1; j < n && key_eq<W>(load_key<W>(keys, j), k); ++j) {
                s = __dadd_rn(s, from_bits(__ldcg(vals + j)));
                if (!is_finite(s)) bad = true;
            }
            out = is_zero(s) ? 0ull : dbits(s);
        }
        sums[i] = out;
    }
    if (bad) atomicOr(status, ST_NUMERIC);
}

// kept[block]: nonzero sums among the block's 1024 entries.
__global__ void __launch_bounds__(kLvBlock) k_lv_kept(const unsigned long long* sums,
                                                     const unsigned long long* count,
                                                     unsigned* kept) {
    __shared__ unsigned s_n;
    if (threadIdx.x == 0) s_n = 0u;
    __syncthreads();
    const unsigned long long n = *count, base = (unsigned long long)blockIdx.x * kLvTile;
    unsigned mine = 0;
#pragma unroll
    for (int e = 0; e < kLvItems; ++e) {
        const unsigned long long i = base + (unsigned long long)e * kLvBlock + threadIdx.x;
        if (i < n && sums[i]) ++mine;
    }
    mine = __reduce_add_sync(0xffffffffu, mine);
    if ((threadIdx.x & 31u) == 0 && mine) atomicAdd(&s_n, mine);
    __syncthreads();
    if (threadIdx.x == 0) kept[blockIdx.x] = s_n;
}

// Writes the nonzero sums, in key order, from offsets[block].
template <int W>
__global__ void __launch_bounds__(kLvBlock) k_lv_write(const uint64_t* keys,
                                                      const unsigned long long* sums,
                                                      const unsigned long long* count,
                                                      const unsigned long long* offsets,
                                                      uint64_t* out_keys, double* out_vals) {
    __shared__ unsigned s_warp[kLvItems][kLvBlock / 32];
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const unsigned long long n = *count, base = (unsigned long long)blockIdx.x * kLvTile;
    bool on[kLvItems];
    unsigned rank[kLvItems];
#pragma unroll
    for (int e = 0; e < kLvItems; ++e) {
        const unsigned long long i = base + (unsigned long long)e * kLvBlock + tid;
        on[e] = i < n && sums[i] != 0ull;
        const unsigned m = __ballot_sync(0xffffffffu, on[e]);
        rank[e] = __popc(m & lanemask_lt());
        if (lane == 0) s_warp[e][warp] = __popc(m);
    }
    __syncthreads();
    unsigned before = 0;
#pragma unroll
    for (int e = 0; e < kLvItems; ++e) {
        unsigned in_round = 0;
        for (unsigned w = 0; w < kLvBlock / 32; ++w) {
            if (w < warp) in_round += s_warp[e][w];
        }
        if (on[e]) {
            const unsigned long long i = base + (unsigned long long)e * kLvBlock + tid;
            const unsigned long long at = offsets[blockIdx.x] + before + in_round + rank[e];
            store_key<W>(out_keys, at, load_key<W>(keys, i));
            reinterpret_cast<unsigned long long*>(out_vals)[at] = sums[i];
        }
        for (unsigned w = 0; w < kLvBlock / 32; ++w) before += s_warp[e][w];
    }
}

}  // namespace tg
