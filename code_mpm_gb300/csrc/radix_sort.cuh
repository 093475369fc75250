// Stable LSD radix sort of (32-bit key, 32-bit value) pairs, DB-bit digits
// (8 to 10; the caller picks the fewest passes that cover the key bits).
//
// Used to order particles by cell key each step.  Stability within a digit
// pass comes from ranking every key against the keys before it in its tile
// (warp match + per-warp digit counters, then a prefix over the warps), so
// equal keys keep their input order; with values 0..n-1 as input the output
// is the particle order of a stable CPU sort by key (std::stable_sort).
//
// Per pass: k_rs_hist (per-tile digit histogram, digit-major layout),
// k_rs_scan (one-block exclusive scan of the histogram), k_rs_scatter.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mpm {

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 16;  // keys per thread
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
constexpr int RS_WARP_TILE = 32 * RS_ITEMS;

template <int DB = 8>
static __global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const unsigned* __restrict__ keys, long long n, int shift,
                                                         unsigned* __restrict__ counts, int nblocks) {
    constexpr unsigned NB = 1u << DB, MASK = NB - 1u;
    __shared__ unsigned h[NB];
    for (int i = threadIdx.x; i < (int)NB; i += RS_THREADS) h[i] = 0;
    __syncthreads();
    long long base = (long long)blockIdx.x * RS_TILE;
#pragma unroll 4
    for (int j = 0; j < RS_ITEMS; ++j) {
        long long idx = base + (long long)j * RS_THREADS + threadIdx.x;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & MASK], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < (int)NB; i += RS_THREADS) counts[(size_t)i * nblocks + blockIdx.x] = h[i];
}

// Exclusive scan of counts[0..total) in place, one block of 1024 threads.
static __global__ void __launch_bounds__(1024) k_rs_scan(unsigned* __restrict__ counts, int total) {
    __shared__ unsigned part[1024];
    const int t = threadIdx.x;
    const int per = (total + 1023) / 1024;
    const int lo = t * per, hi = min(total, lo + per);
    unsigned s = 0;
    for (int i = lo; i < hi; ++i) s += counts[i];
    part[t] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        unsigned v = (t >= off) ? part[t - off] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    unsigned run = part[t] - s;  // exclusive prefix of this thread's chunk
    for (int i = lo; i < hi; ++i) {
        unsigned c = counts[i];
        counts[i] = run;
        run += c;
    }
}

// Two-level exclusive scan of the histogram for large inputs: k_rs_scan_chunks
// scans RS_SCAN_CHUNK entries per block in place and records each chunk's
// total; k_rs_scan (one block) then scans the chunk totals; the scatter adds
// the chunk prefix to every offset it reads.
constexpr int RS_SCAN_THREADS = 1024;
constexpr int RS_SCAN_PER_THREAD = 4;
constexpr int RS_SCAN_CHUNK = RS_SCAN_THREADS * RS_SCAN_PER_THREAD;

static __global__ void __launch_bounds__(RS_SCAN_THREADS) k_rs_scan_chunks(unsigned* __restrict__ counts, int total,
                                                                          unsigned* __restrict__ chunk_totals) {
    __shared__ unsigned wsum[RS_SCAN_THREADS / 32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const long long base = (long long)blockIdx.x * RS_SCAN_CHUNK + (long long)t * RS_SCAN_PER_THREAD;
    unsigned v[RS_SCAN_PER_THREAD], s = 0;
#pragma unroll
    for (int j = 0; j < RS_SCAN_PER_THREAD; ++j) {
        v[j] = (base + j < total) ? counts[base + j] : 0u;
        s += v[j];
    }
    unsigned inc = s;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        unsigned o = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= d) inc += o;
    }
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    if (w == 0) {
        unsigned x = wsum[lane];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            unsigned o = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += o;
        }
        wsum[lane] = x;  // inclusive over warps
    }
    __syncthreads();
    unsigned run = inc - s + (w > 0 ? wsum[w - 1] : 0u);
#pragma unroll
    for (int j = 0; j < RS_SCAN_PER_THREAD; ++j) {
        if (base + j < total) counts[base + j] = run;
        run += v[j];
    }
    if (t == RS_SCAN_THREADS - 1) chunk_totals[blockIdx.x] = wsum[31];
}

template <int DB = 8>
static __global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const unsigned* __restrict__ kin,
                                                            const unsigned* __restrict__ vin,
                                                            unsigned* __restrict__ kout, unsigned* __restrict__ vout,
                                                            long long n, int shift,
                                                            const unsigned* __restrict__ offs, int nblocks,
                                                            const unsigned* __restrict__ chunk_prefix) {
    constexpr unsigned NB = 1u << DB, MASK = NB - 1u;
    __shared__ unsigned wcnt[RS_WARPS][NB];
    __shared__ unsigned gofs[NB];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < RS_WARPS * (int)NB; i += RS_THREADS) (&wcnt[0][0])[i] = 0;
    for (int i = threadIdx.x; i < (int)NB; i += RS_THREADS) {
        size_t j = (size_t)i * nblocks + blockIdx.x;
        gofs[i] = offs[j] + (chunk_prefix ? chunk_prefix[j / RS_SCAN_CHUNK] : 0u);
    }
    __syncthreads();
    const long long base = (long long)blockIdx.x * RS_TILE + (long long)w * RS_WARP_TILE;
    const unsigned lt = (1u << lane) - 1u;
    unsigned k[RS_ITEMS], v[RS_ITEMS], r[RS_ITEMS];
#pragma unroll
    for (int c = 0; c < RS_ITEMS; ++c) {
        long long idx = base + c * 32 + lane;
        bool ok = idx < n;
        unsigned key = ok ? kin[idx] : 0u;
        unsigned val = ok ? (vin ? vin[idx] : (unsigned)idx) : 0u;  // no input values: the identity
        unsigned d = ok ? ((key >> shift) & MASK) : (NB + lane);  // invalid lanes never match a digit
        unsigned peers = __match_any_sync(0xffffffffu, d);
        unsigned rank = 0;
        if (ok) rank = wcnt[w][d] + __popc(peers & lt);
        __syncwarp();
        if (ok && lane == __ffs(peers) - 1) wcnt[w][d] += __popc(peers);
        __syncwarp();
        k[c] = key;
        v[c] = val;
        r[c] = rank;
    }
    __syncthreads();
    for (int d = threadIdx.x; d < (int)NB; d += RS_THREADS) {
        unsigned run = 0;
        for (int ww = 0; ww < RS_WARPS; ++ww) {
            unsigned t = wcnt[ww][d];
            wcnt[ww][d] = run;
            run += t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < RS_ITEMS; ++c) {
        long long idx = base + c * 32 + lane;
        if (idx < n) {
            unsigned d = (k[c] >> shift) & MASK;
            unsigned dst = gofs[d] + wcnt[w][d] + r[c];
            kout[dst] = k[c];
            vout[dst] = v[c];
        }
    }
}

}  // namespace mpm
