// The FP32 form's scatter kernels with the run reduction in registers and
// warp shuffles (P2G modes 5 and 6): P2G (M2G, …MPLocks.cpp:48-89, and the
// contact path's mass gradient, …_Contact.cpp:131) and G2P pass 1 with the
// velocity remap (:489-510, :539-564).
//
// A block of BS threads takes a tile of TS = 4 BS consecutive slots.  The
// tile's runs of equal cell keys (a cell's particles, adjacent in cell order;
// a cell met twice is two runs) are found in shared memory.  Each run goes to
// a pair of adjacent lanes that split its particles (even and odd places in
// the run); each lane reads each of its particles once and forms all eight
// corners' seven sums (mass, momentum, force) in registers.  One shuffle
// exchange between the two lanes then leaves the even lane with the sums of
// the four corners at ix = 0 and the odd lane with those at ix = 1, and each
// lane adds its four corners to the nodes with two vector atomics per corner.
// So every particle is read once, nothing is staged for a scatter pass, and
// the only reduction before the global atomics is the warp shuffle.
//
// Mode 6 brings the tile's particle fields (cell-local coordinate, mass,
// volume, velocity, stress, external force: 17 float segments) into shared
// memory first, with bulk copies (cp.async.bulk) issued by one warp and
// completed on one mbarrier, so a lane's reads wait for one memory round trip
// instead of one per particle; the run finding overlaps the copies.  Tiles
// that cannot stage (the last one, unaligned arrays, a sort permutation)
// read global memory like mode 5.
#pragma once

#include "kernels.cuh"

namespace mpm {

constexpr int PAIR_TILE_PER_THREAD = 4;  // slots per thread in a tile

// The tile's runs: run r covers tile slots run_start[r] .. run_start[r + 1] - 1
// (keys in skey for the tile's first nslots slots).  Thread t looks at slots
// 4t .. 4t + 3.  Returns the run count.
template <int BS>
__device__ __forceinline__ int tile_runs(const unsigned* skey, int nslots, int* run_start, int* wsum) {
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    unsigned hm = 0u;
#pragma unroll
    for (int j = 0; j < PAIR_TILE_PER_THREAD; ++j) {
        const int i = PAIR_TILE_PER_THREAD * t + j;
        const bool head = i < nslots && (i == 0 || skey[i - 1] != skey[i]);
        hm |= (head ? 1u : 0u) << j;
    }
    const int h = __popc(hm);
    int incl = h;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int o = __shfl_up_sync(FULL_MASK, incl, off);
        if (lane >= off) incl += o;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    if (t < 32) {
        constexpr int NW = BS / 32;
        const int v = (t < NW) ? wsum[t] : 0;
        int x = v;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int o = __shfl_up_sync(FULL_MASK, x, off);
            if (t >= off) x += o;
        }
        if (t < NW) wsum[t] = x - v;
        if (t == 31) wsum[32] = x;
    }
    __syncthreads();
    int at = wsum[w] + incl - h;
#pragma unroll
    for (int j = 0; j < PAIR_TILE_PER_THREAD; ++j)
        if ((hm >> j) & 1u) run_start[at++] = PAIR_TILE_PER_THREAD * t + j;
    const int R = wsum[32];
    if (t == 0) run_start[R] = nslots;
    __syncthreads();
    return R;
}

// The 17 particle-field segments of a tile (float each): 0-2 cell-local
// coordinate, 3 mass, 4 volume, 5-7 velocity, 8-13 stress, 14-16 external
// force.  Segment i is component k of array base.
__device__ __forceinline__ const float* pair_segment(int i, const PView<float>& P, int& k) {
    if (i < 3) {
        k = i;
        return P.loc;
    }
    if (i == 3) {
        k = 0;
        return P.mass;
    }
    if (i == 4) {
        k = 0;
        return P.vol;
    }
    if (i < 8) {
        k = i - 5;
        return P.vel;
    }
    if (i < 14) {
        k = i - 8;
        return P.stress;
    }
    k = i - 14;
    return P.fext;
}

// A tile's segments in shared memory: TS floats plus 16 bytes each, copied
// from the 16-byte boundary at or below the tile's first element (element j
// of component k sits ((k n + s0) mod 4) floats into its segment).  Usable
// when every array starts on a 16-byte boundary and s0 + TS + 4 <= n (the
// copies then stay inside their arrays).
template <int TS>
struct PairStage {
    static constexpr int NSEG = 17;
    static constexpr int SEG = TS * 4 + 16;
    static constexpr int BYTES = NSEG * SEG;

    static __device__ __forceinline__ bool usable(const PView<float>& P, long long s0, long long n) {
        const unsigned long long a = (unsigned long long)P.loc | (unsigned long long)P.mass |
                                     (unsigned long long)P.vol | (unsigned long long)P.vel |
                                     (unsigned long long)P.stress | (unsigned long long)P.fext;
        return P.loc && P.mass && P.vol && P.vel && P.stress && P.fext && (a & 15ull) == 0 && s0 + TS + 4 <= n;
    }
    static __device__ __forceinline__ void copy(int i, const PView<float>& P, long long s0, unsigned char* sm,
                                                uint32_t bar) {
        int k;
        const float* base = pair_segment(i, P, k);
        const unsigned long long src = (unsigned long long)(base + (long long)k * P.n + s0) & ~15ull;
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                shared_addr(sm + i * SEG)),
            "l"(src), "r"((unsigned)SEG), "r"(bar)
            : "memory");
    }
};

// Where a lane reads particle fields from: global memory at the particle's
// index, or the staged tile at the slot's place in it.
struct PairDirect {
    const PView<float>* P;
    __device__ __forceinline__ float get(int i, int, long long p) const {
        int k;
        const float* base = pair_segment(i, *P, k);
        return base[(long long)k * P->n + p];
    }
};

template <int TS>
struct PairStaged {
    const unsigned char* sm;
    int nm, s0m;  // n mod 4, s0 mod 4: the misalignment of component k is ((k n + s0) mod 4) floats
    __device__ __forceinline__ float get(int i, int j, long long) const {
        const int k = i < 3 ? i : (i < 5 ? 0 : (i < 8 ? i - 5 : (i < 14 ? i - 8 : i - 14)));
        const int mis = (k * nm + s0m) & 3;
        return reinterpret_cast<const float*>(sm + i * PairStage<TS>::SEG)[mis + j];
    }
};

// Sum one run's share of particles (tile slots a + par, a + par + 2, ... < e)
// into the eight corners' sums.  Products as in the cell-run P2G, regrouped
// around the z factor: with A = Nx Ny, Bx = Ny gx, By = Nx gy a corner's
// N = A Nz and G = -(Bx Nz, By Nz, A gz), so its force is Nz c + gz d with
// c and d formed once per particle and (x, y) pair.
template <bool MG, class SRC>
__device__ __forceinline__ void pair_accumulate(const SRC& src, const unsigned* __restrict__ perm, long long s0,
                                                int a, int e, int par, const Geom& gs, float am[8], float ap0[8],
                                                float ap1[8], float ap2[8], float af0[8], float af1[8],
                                                float af2[8], float g0[8], float g1[8], float g2[8]) {
    for (int j = a + par; j < e; j += 2) {
        const long long p = perm ? (long long)perm[s0 + j] : s0 + j;
        float Nx[2], gx[2], Ny[2], gy[2], Nz[2], gz[2];
        axis_bases_u(src.get(0, j, p), gs.inv_hf[0], Nx, gx);
        axis_bases_u(src.get(1, j, p), gs.inv_hf[1], Ny, gy);
        axis_bases_u(src.get(2, j, p), gs.inv_hf[2], Nz, gz);
        const float m = src.get(3, j, p), V = src.get(4, j, p);
        const float mv0 = m * src.get(5, j, p), mv1 = m * src.get(6, j, p), mv2 = m * src.get(7, j, p);
        const float v0 = -V * src.get(8, j, p), v1 = -V * src.get(9, j, p), v2 = -V * src.get(10, j, p);
        const float v3 = -V * src.get(11, j, p), v4 = -V * src.get(12, j, p), v5 = -V * src.get(13, j, p);
        const float fe0 = src.get(14, j, p), fe1 = src.get(15, j, p), fe2 = src.get(16, j, p);
#pragma unroll
        for (int ix = 0; ix < 2; ++ix)
#pragma unroll
            for (int iy = 0; iy < 2; ++iy) {
                const float A = Nx[ix] * Ny[iy], Bx = Ny[iy] * gx[ix], By = Nx[ix] * gy[iy];
                const float Am = A * m, Am0 = A * mv0, Am1 = A * mv1, Am2 = A * mv2;
                const float c0 = A * fe0 - Bx * v0 - By * v3;
                const float c1 = A * fe1 - By * v1 - Bx * v3;
                const float c2 = A * fe2 - Bx * v5 - By * v4;
                const float d0 = -A * v5, d1 = -A * v4, d2 = -A * v2;
#pragma unroll
                for (int iz = 0; iz < 2; ++iz) {
                    const int k = 4 * ix + 2 * iy + iz;
                    const float nz = Nz[iz], gzv = gz[iz];
                    am[k] += nz * Am;
                    ap0[k] += nz * Am0;
                    ap1[k] += nz * Am1;
                    ap2[k] += nz * Am2;
                    af0[k] = fmaf(gzv, d0, fmaf(nz, c0, af0[k]));
                    af1[k] = fmaf(gzv, d1, fmaf(nz, c1, af1[k]));
                    af2[k] = fmaf(gzv, d2, fmaf(nz, c2, af2[k]));
                    if constexpr (MG) {
                        g0[k] -= nz * (Bx * m);
                        g1[k] -= nz * (By * m);
                        g2[k] -= gzv * Am;
                    }
                }
            }
    }
}

// The pair exchange: the even lane keeps corners 0-3 (ix = 0), the odd lane
// corners 4-7 (ix = 1); each sends the other half and adds what it receives.
__device__ __forceinline__ void pair_exchange(float v[8], int par) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float send = par ? v[j] : v[4 + j];
        const float keep = par ? v[4 + j] : v[j];
        v[j] = keep + __shfl_xor_sync(FULL_MASK, send, 1);
    }
}

template <int BS, bool MG, bool STAGE>
__global__ void __launch_bounds__(BS) k_p2g_pairs(PView<float> P, NView<float> nd, Geom g,
                                                   const unsigned* __restrict__ skeys,
                                                   const unsigned* __restrict__ perm, long long n, int mark_active,
                                                   unsigned* err) {
    constexpr int TS = PAIR_TILE_PER_THREAD * BS;
    using S = PairStage<TS>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char* stage = smem_raw;  // S::BYTES when staging
    unsigned* skey = reinterpret_cast<unsigned*>(smem_raw + (STAGE ? S::BYTES : 0));
    int* run_start = reinterpret_cast<int*>(skey + TS);  // TS + 1
    int* wsum = run_start + TS + 1;                       // 33
    unsigned long long* bar_mem = reinterpret_cast<unsigned long long*>(smem_raw + (STAGE ? S::BYTES : 0) +
                                                                         ((size_t)TS * 8 + 4 + 33 * 4 + 15) / 16 * 16);
    const int t = threadIdx.x, lane = t & 31;
    const long long s0 = blockIdx.x * (long long)TS;
    const int nslots = (int)min((long long)TS, n - s0);
    const bool staged = STAGE && perm == nullptr && S::usable(P, s0, n);
    const uint32_t bar = shared_addr(bar_mem);
    if (staged) {
        if (t == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
        __syncthreads();
        if (t < 32) {
            if (t == 0)
                asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n" ::"r"(bar),
                             "r"((unsigned)S::BYTES)
                             : "memory");
            __syncwarp();
            for (int i = t; i < S::NSEG; i += 32) S::copy(i, P, s0, stage, bar);
        }
    }
    // the tile's keys (storage order), then its runs, while the copies are in flight
#pragma unroll
    for (int j = 0; j < PAIR_TILE_PER_THREAD; ++j) {
        const int i = j * BS + t;
        skey[i] = (i < nslots) ? skeys[s0 + i] : 0xffffffffu;
    }
    __syncthreads();
    const int R = tile_runs<BS>(skey, nslots, run_start, wsum);
    if (staged && !mbar_wait(bar, 0, err)) {
        mbar_wait(bar, 0, err);  // once more (bounded) for copies still in flight, then leave
        return;
    }
    const long long nn = nd.nn;
    // every lane of a warp runs the same number of rounds (the shuffles take the full warp)
    for (int base = t - lane; base < 2 * R; base += BS) {
        const int item = base + lane, par = item & 1;
        const bool live = item < 2 * R;
        float am[8], ap0[8], ap1[8], ap2[8], af0[8], af1[8], af2[8], g0[8], g1[8], g2[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) am[k] = ap0[k] = ap1[k] = ap2[k] = af0[k] = af1[k] = af2[k] = g0[k] = g1[k] = g2[k] = 0.0f;
        int a = 0, e = 0;
        unsigned key = 0xffffffffu;
        if (live) {
            a = run_start[item >> 1];
            e = run_start[(item >> 1) + 1];
            key = skey[a];
        }
        const bool valid = key < g.key_max;
        const Geom* gsp = &g;
        if (valid) {
            gsp = &spec_geom(g, P.sid, perm ? (long long)perm[s0 + a] : s0 + a);
            if (staged)
                pair_accumulate<MG>(PairStaged<TS>{stage, (int)(P.n & 3), (int)(s0 & 3)}, perm, s0, a, e, par, *gsp,
                                    am, ap0, ap1, ap2, af0, af1, af2, g0, g1, g2);
            else
                pair_accumulate<MG>(PairDirect{&P}, perm, s0, a, e, par, *gsp, am, ap0, ap1, ap2, af0, af1, af2, g0,
                                    g1, g2);
        }
        pair_exchange(am, par);
        pair_exchange(ap0, par);
        pair_exchange(ap1, par);
        pair_exchange(ap2, par);
        pair_exchange(af0, par);
        pair_exchange(af1, par);
        pair_exchange(af2, par);
        if constexpr (MG) {
            pair_exchange(g0, par);
            pair_exchange(g1, par);
            pair_exchange(g2, par);
        }
        if (!valid) continue;
        int b[3];
        key_to_base(key, *gsp, b);
        const CellNodes cn = cell_nodes(*gsp, b);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int k = 4 * par + j;
            if (!((cn.mask >> k) & 1u)) continue;
            const long long nid = cell_node(cn, k);
            // active nodes: the in-range corners of occupied cells (b_Active, …MPLocks.cpp:36)
            if (mark_active) atomicOr(&nd.state[nid], 1u);
            acc_add<float>(nd.acc, nid, am[j], ap0[j], ap1[j], ap2[j], af0[j], af1[j], af2[j]);
            if constexpr (MG) {
                atomicAdd(&nd.mg[nid], g0[j]);
                atomicAdd(&nd.mg[nn + nid], g1[j]);
                atomicAdd(&nd.mg[2 * nn + nid], g2[j]);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// G2P pass 1 + velocity remap over the same runs (P2G modes 5 and 6).  A run's
// particles share one cell, so each lane of the run's pair loads the cell's
// eight node records {f/m, m > m_min} once, then for each of its particles
// adds N (f/m) dt over the corners in corner order (the velocity update of
// …MPLocks.cpp:489-510) and forms N m v for the eight corners (:539-564); the
// pair exchange leaves each lane four corners' remap sums, one vector atomic
// each.  Particles skipped on the contact path (b_DisplacementControl) keep
// their velocity and add nothing.
// ---------------------------------------------------------------------------
template <int BS>
__global__ void __launch_bounds__(BS) k_pass1_pairs(PView<float> P, NView<float> nd, Geom g,
                                                     const unsigned* __restrict__ skeys,
                                                     const unsigned* __restrict__ perm, long long n, float dt,
                                                     int contact) {
    constexpr int TS = PAIR_TILE_PER_THREAD * BS;
    __shared__ unsigned skey[TS];
    __shared__ int run_start[TS + 1];
    __shared__ int wsum[33];
    const int t = threadIdx.x, lane = t & 31;
    const long long s0 = blockIdx.x * (long long)TS;
    const int nslots = (int)min((long long)TS, n - s0);
#pragma unroll
    for (int j = 0; j < PAIR_TILE_PER_THREAD; ++j) {
        const int i = j * BS + t;
        skey[i] = (i < nslots) ? skeys[s0 + i] : 0xffffffffu;
    }
    __syncthreads();
    const int R = tile_runs<BS>(skey, nslots, run_start, wsum);
    const long long np = P.n;
    for (int base = t - lane; base < 2 * R; base += BS) {
        const int item = base + lane, par = item & 1;
        const bool live = item < 2 * R;
        float q0[8], q1[8], q2[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) q0[k] = q1[k] = q2[k] = 0.0f;
        int a = 0, e = 0;
        unsigned key = 0xffffffffu;
        if (live) {
            a = run_start[item >> 1];
            e = run_start[(item >> 1) + 1];
            key = skey[a];
        }
        const bool valid = key < g.key_max;
        CellNodes cn;
        cn.mask = 0u;
        if (valid) {
            const Geom& gs = spec_geom(g, P.sid, perm ? (long long)perm[s0 + a] : s0 + a);
            int b[3];
            key_to_base(key, gs, b);
            cn = cell_nodes(gs, b);
            Quad<float> rq[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const Quad<float> z{0.0f, 0.0f, 0.0f, 0.0f};
                rq[k] = ((cn.mask >> k) & 1u) ? ld_quad(nd.rec + 8 * cell_node(cn, k)) : z;
            }
            for (int j = a + par; j < e; j += 2) {
                const long long p = perm ? (long long)perm[s0 + j] : s0 + j;
                if (contact && (P.pflags[p] & 8u)) continue;
                float Nx[2], gx[2], Ny[2], gy[2], Nz[2], gz[2];
                axis_bases_u(P.loc[p], gs.inv_hf[0], Nx, gx);
                axis_bases_u(P.loc[np + p], gs.inv_hf[1], Ny, gy);
                axis_bases_u(P.loc[2 * np + p], gs.inv_hf[2], Nz, gz);
                float v[3] = {P.vel[p], P.vel[np + p], P.vel[2 * np + p]};
                const float m = P.mass[p];
                float Nk[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    Nk[k] = Nx[(k >> 2) & 1] * Ny[(k >> 1) & 1] * Nz[k & 1];
                    if (!(rq[k].w != 0.0f)) continue;  // out of range or m <= mass_min
                    v[0] = v[0] + Nk[k] * rq[k].x * dt;
                    v[1] = v[1] + Nk[k] * rq[k].y * dt;
                    v[2] = v[2] + Nk[k] * rq[k].z * dt;
                }
#pragma unroll
                for (int c = 0; c < 3; ++c) P.vel[c * np + p] = v[c];
                const float mv0 = m * v[0], mv1 = m * v[1], mv2 = m * v[2];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    q0[k] += Nk[k] * mv0;
                    q1[k] += Nk[k] * mv1;
                    q2[k] += Nk[k] * mv2;
                }
            }
        }
        pair_exchange(q0, par);
        pair_exchange(q1, par);
        pair_exchange(q2, par);
        if (!valid) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int k = 4 * par + j;
            if ((cn.mask >> k) & 1u) q_add<float>(nd.q, cell_node(cn, k), q0[j], q1[j], q2[j]);
        }
    }
}

// Dynamic shared memory of k_p2g_pairs: the staged segments (mode 6), the
// tile's keys, run starts and warp counts, the mbarrier.
template <int BS>
constexpr size_t p2g_pairs_smem(bool stage) {
    return (stage ? (size_t)PairStage<PAIR_TILE_PER_THREAD * BS>::BYTES : 0) +
           ((size_t)PAIR_TILE_PER_THREAD * BS * 8 + 4 + 33 * 4 + 15) / 16 * 16 + 16;
}

}  // namespace mpm
