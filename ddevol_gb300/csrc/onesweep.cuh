// Stable LSD radix sort of (key, value) pairs by multi-word key, onesweep
// style: one pass computes the histograms of every 8-bit digit, then one
// scatter pass per digit finds each tile's output offsets by a decoupled
// look-back over the tiles before it (per digit bucket) and writes the tile
// through shared memory so that each bucket's run leaves as consecutive
// addresses.  Keys are the map's multi-word keys (highest word most
// significant); digit d covers bits 8d..8d+7 of the 2N used bits, so
// ceil(2N / 8) passes sort completely and stably.
//
// The item count is read from device memory (so a captured graph serves any
// count) and clamped to the buffers' capacity; every look-back wait is
// bounded (ST_TIMEOUT) and a set status word makes every kernel return at
// once.
#pragma once
#include "common.cuh"

namespace tg {

constexpr int kOsBlock = 256, kOsItems = 8, kOsTile = kOsBlock * kOsItems;
constexpr int kOsMaxDigits = 32;  // keys of up to 128 spins (four words)
constexpr unsigned long long kOsAgg = 1ull << 62, kOsPre = 2ull << 62;
constexpr unsigned long long kOsCount = (1ull << 62) - 1;

struct SortArgs {
    const unsigned long long* count;  // items to sort (device), clamped to cap
    unsigned long long cap;           // capacity of every buffer, in items
    unsigned* status;                 // nonzero: return at once; ST_TIMEOUT on a lost wait
    unsigned long long* hist;         // [digits][256] counts, then exclusive bucket bases
    unsigned long long* look;         // [tiles][256] look-back words of the current pass
    unsigned* tile_counter;           // tiles handed out in the current pass
    const unsigned long long* expect; // NULL, or the count the producer reported (must match)
    const unsigned* wait_polls;       // NULL or 0: the default look-back poll limit
    int digits;
};

template <int W>
__device__ __forceinline__ unsigned sort_digit(const Key<W>& k, int d) {
    return (unsigned)((word_at<W>(k, d >> 3) >> ((d & 7) * 8)) & 0xffull);
}

__device__ __forceinline__ unsigned long long sort_count(const SortArgs& a) {
    return min(*reinterpret_cast<const volatile unsigned long long*>(a.count), a.cap);
}

// Histograms of all digits: per-CTA counts in shared memory, then added.
template <int W>
__global__ void __launch_bounds__(kOsBlock) k_os_hist(const uint64_t* keys, SortArgs a) {
    __shared__ unsigned s_h[kOsMaxDigits][256];
    if (*reinterpret_cast<const volatile unsigned*>(a.status)) return;
    const int D = a.digits;
    for (int q = threadIdx.x; q < D * 256; q += blockDim.x) (&s_h[0][0])[q] = 0u;
    __syncthreads();
    const unsigned long long n = sort_count(a);
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += stride) {
        const Key<W> k = load_key<W>(keys, i);
        for (int d = 0; d < D; ++d) atomicAdd(&s_h[d][sort_digit<W>(k, d)], 1u);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < D * 256; q += blockDim.x) {
        const unsigned v = (&s_h[0][0])[q];
        if (v) atomicAdd(a.hist + q, (unsigned long long)v);
    }
}

// Exclusive bucket bases of every digit (one CTA of 256 threads).
__global__ void __launch_bounds__(256) k_os_bases(SortArgs a) {
    __shared__ unsigned long long s_v[256];
    if (*reinterpret_cast<const volatile unsigned*>(a.status)) return;
    if (a.expect && threadIdx.x == 0 && *a.expect != sort_count(a)) atomicOr(a.status, ST_ORDER);
    for (int d = 0; d < a.digits; ++d) {
        const unsigned long long mine = a.hist[d * 256 + threadIdx.x];
        s_v[threadIdx.x] = mine;
        __syncthreads();
        for (int off = 1; off < 256; off <<= 1) {
            const unsigned long long v = threadIdx.x >= (unsigned)off ? s_v[threadIdx.x - off] : 0ull;
            __syncthreads();
            s_v[threadIdx.x] += v;
            __syncthreads();
        }
        a.hist[d * 256 + threadIdx.x] = s_v[threadIdx.x] - mine;
        __syncthreads();
    }
}

template <int W>
constexpr size_t os_smem() {
    return (size_t)kOsTile * (8 * W + 8);
}

// One stable scatter pass for digit d: sk/sv -> dk/dv (dk == nullptr: the
// destination named in *out_keys / *out_vals, read at run time).
template <int W>
__global__ void __launch_bounds__(kOsBlock) k_os_scatter(const uint64_t* sk,
                                                        const unsigned long long* sv, uint64_t* dk,
                                                        unsigned long long* dv,
                                                        uint64_t* const* out_keys,
                                                        double* const* out_vals, SortArgs a, int d) {
    extern __shared__ __align__(16) unsigned char os_raw[];
    uint64_t* st_k = reinterpret_cast<uint64_t*>(os_raw);                      // [tile][W]
    unsigned long long* st_v = reinterpret_cast<unsigned long long*>(st_k + (size_t)kOsTile * W);
    __shared__ unsigned s_cnt[256], s_local[256], s_run[256];
    __shared__ unsigned long long s_gbase[256];
    __shared__ unsigned s_w[kOsBlock / 32][256];
    __shared__ unsigned s_tile;
    if (*reinterpret_cast<const volatile unsigned*>(a.status)) return;
    if (!dk) {
        dk = *out_keys;
        dv = reinterpret_cast<unsigned long long*>(*out_vals);
    }
    const unsigned long long n = sort_count(a);
    const unsigned long long ntiles = (n + kOsTile - 1) / kOsTile;
    const unsigned long long* base_d = a.hist + (size_t)d * 256;
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    for (;;) {
        __syncthreads();
        if (tid == 0) s_tile = atomicAdd(a.tile_counter, 1u);
        s_cnt[tid] = 0u;
        s_run[tid] = 0u;
        __syncthreads();
        const unsigned long long tile = s_tile;
        if (tile >= ntiles) break;
        const unsigned long long t0 = tile * kOsTile;
        // load the tile (round e: items t0 + 256 e + tid) and count its digits
        Key<W> key[kOsItems];
        unsigned long long val[kOsItems];
        unsigned dig[kOsItems];
#pragma unroll
        for (int e = 0; e < kOsItems; ++e) {
            const unsigned long long i = t0 + (unsigned long long)e * kOsBlock + tid;
            dig[e] = 256u;
            if (i < n) {
                key[e] = load_key<W>(sk, i);
                val[e] = __ldcg(sv + i);
                dig[e] = sort_digit<W>(key[e], d);
                atomicAdd(&s_cnt[dig[e]], 1u);
            }
        }
        __syncthreads();
        // bucket tid: publish the tile's count, look back for the prefix
        {
            const unsigned long long mine = s_cnt[tid];
            unsigned long long* slot = a.look + tile * 256 + tid;
            unsigned long long excl = 0;
            if (tile == 0) {
                publish(slot, kOsPre | mine);
            } else {
                publish(slot, kOsAgg | mine);
                long long t = (long long)tile - 1;
                unsigned polls = 0, limit = kLookbackPolls;
                if (a.wait_polls && *a.wait_polls) limit = *a.wait_polls;
                while (t >= 0) {
                    unsigned long long w = poll(a.look + (unsigned long long)t * 256 + tid);
                    while (!(w >> 62)) {
                        if (++polls > limit) {
                            atomicOr(a.status, ST_TIMEOUT);
                            w = kOsPre;  // give up: an empty prefix
                            break;
                        }
                        w = poll(a.look + (unsigned long long)t * 256 + tid);
                    }
                    excl += w & kOsCount;
                    if ((w >> 62) == 2) break;
                    --t;
                }
                publish(slot, kOsPre | (excl + mine));
            }
            s_gbase[tid] = base_d[tid] + excl;
        }
        // exclusive scan of the tile's counts: local bucket offsets
        {
            unsigned v = s_cnt[tid];
            s_local[tid] = v;
            __syncthreads();
            for (int off = 1; off < 256; off <<= 1) {
                const unsigned x = tid >= (unsigned)off ? s_local[tid - off] : 0u;
                __syncthreads();
                s_local[tid] += x;
                __syncthreads();
            }
            s_local[tid] -= v;
        }
        // stable ranks (round, warp, lane order = index order) into the stage
#pragma unroll
        for (int e = 0; e < kOsItems; ++e) {
            for (int q = lane; q < 256; q += 32) s_w[warp][q] = 0u;
            __syncthreads();
            const unsigned peers = __match_any_sync(0xffffffffu, dig[e]);
            if (dig[e] < 256u && lane == (unsigned)(__ffs(peers) - 1)) s_w[warp][dig[e]] = __popc(peers);
            __syncthreads();
            if (dig[e] < 256u) {
                unsigned before = 0;
                for (unsigned w = 0; w < warp; ++w) before += s_w[w][dig[e]];
                const unsigned pos = s_local[dig[e]] + s_run[dig[e]] + before + __popc(peers & lanemask_lt());
#pragma unroll
                for (int w = 0; w < W; ++w) st_k[(size_t)pos * W + w] = key[e].w[w];
                st_v[pos] = val[e];
            }
            __syncthreads();
            unsigned tot = 0;
#pragma unroll
            for (int w = 0; w < kOsBlock / 32; ++w) tot += s_w[w][tid];
            s_run[tid] += tot;
            __syncthreads();  // every row read before the next round clears it
        }
        __syncthreads();
        // write out: consecutive stage slots of one bucket go to consecutive addresses
        const unsigned len = (unsigned)min((unsigned long long)kOsTile, n - t0);
        for (unsigned q = tid; q < len; q += kOsBlock) {
            Key<W> k;
#pragma unroll
            for (int w = 0; w < W; ++w) k.w[w] = st_k[(size_t)q * W + w];
            const unsigned b = sort_digit<W>(k, d);
            const unsigned long long to = s_gbase[b] + (q - s_local[b]);
            if (to < a.cap) {
                store_key<W>(dk, to, k);
                dv[to] = st_v[q];
            } else {
                atomicOr(a.status, ST_ORDER);
            }
        }
    }
}

}  // namespace tg
