// Step kernels of the GB300 MPM engine.  One step of the reference's
// double-pass loop (PhysicsEngine_runSimulation_Classic_DoublePass_MPLocks.cpp:462-792,
// contact variant PhysicsEngine_runSimulation_Classic_DoublePass_MPLocks_Contact.cpp:27-543)
// maps onto:
//   k_reset_grid        ResetGrid (:4-22)
//   k_cell_keys         FindAGPs cell lookup, floor(x/h) (GridPoint_Mediator.cpp:8)
//   radix sort          particles ordered by cell key
//   k_cell_ranges       active-node marking (b_Active, :36) + per-cell particle ranges
//   k_p2g               M2G (:48-89): warp-segmented reduction, then one atomic per run
//   k_dc_claim          DisplacementControl (:143-174), last writer in list order
//   k_node_phase_a      displacement control, IntegrateGrid (:90-142; contact :242-277),
//                       f/m per node (the divisor of G2P pass 1)
//   k_pass1_remap       G2P pass 1 (:489-510) fused with the velocity remap (:539-564)
//   k_node_phase_b      v_i += (sum N m_p v_p) / m_i, displacement control, BC reapply
//                       (:573-599), p/m and v per node
//   k_pass2             G2P_P2_SmallStrain (:175-280; contact :438-525) fused with the
//                       constitutive increment and the platen timeline (:766-789)
//   k_contact_*         contact detection (…_Contact.cpp:152-237), bit-exact
#pragma once

#include "common.cuh"
#include "physics.cuh"
#include "surrogate.cuh"

namespace mpm {

// ---------------------------------------------------------------------------
// grid reset: zero every node that was active (the reference only clears
// active nodes; inactive ones are already zero).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_reset_grid(NView<T> nd, int contact) {
    const long long nn = nd.nn;
    NODE_LOOP(nd, i) {
        unsigned st = nd.state[i];
        if (!(st & 1u)) continue;
        nd.state[i] = contact ? 0u : (st & ~(1u | NODE_CLAIMED));
        const Quad<T> z{(T)0, (T)0, (T)0, (T)0};
        *reinterpret_cast<Quad<T>*>(nd.acc + 8 * i) = z;
        *reinterpret_cast<Quad<T>*>(nd.acc + 8 * i + 4) = z;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (contact) nd.mg[c * nn + i] = 0.0;
            nd.vel[c * nn + i] = (T)0;
            nd.ftemp[c * nn + i] = (T)0;
        }
    }
}

// ---------------------------------------------------------------------------
// cell keys: base cell b = floor(x/h) per axis with the correctly rounded
// quotient, as glm::floor(d3Position / d3_Length_Cell)
// (GridPoint_Mediator.cpp:8), so the cell index is bit-identical to the
// reference.  Particles whose base cell lies outside [-1, cells] have no node
// in range and get key_max.  Decided in float-float arithmetic (fps_cell)
// unless the quotient lies within 1e-4 of an integer, then by the exact FP64
// quotient (cell_and_local).
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned particle_key(const Geom& g, const double x[3], float u[3], unsigned* err) {
    bool ok = true;
    int b[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float ff;
        if (fps_cell(x[a], g.inv_hf[a], g.ih_lo[a], &ff, &u[a])) {
            if (ff < -1.0f || ff > (float)(g.nn[a] - 1)) ok = false;
            b[a] = ok ? (int)ff : 0;
            continue;
        }
        double f;
        if (!cell_and_local(g, a, x[a], f, u[a])) {
            atomicOr(err, ERR_NONFINITE_POSITION);
            ok = false;
            b[a] = 0;
            continue;
        }
        if (f < -1.0 || f > (double)(g.nn[a] - 1)) ok = false;
        b[a] = ok ? (int)f : 0;
    }
    return ok ? g.key_off + (unsigned)((b[0] + 1) + g.kd[0] * ((b[1] + 1) + g.kd[1] * (b[2] + 1))) : g.key_max;
}

static __global__ void k_cell_keys(const double* __restrict__ pos, long long n, Geom g, unsigned* __restrict__ keys,
                            unsigned* __restrict__ vals, unsigned* __restrict__ keys_copy, unsigned* err,
                            float* __restrict__ loc, const uint16_t* __restrict__ sid) {
    long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= n) return;
    const double x[3] = {pos[p], pos[n + p], pos[2 * n + p]};
    float u[3];
    const unsigned key = particle_key(spec_geom(g, sid, p), x, u, err);
    keys[p] = key;
    keys_copy[p] = key;
    if (vals) vals[p] = (unsigned)p;
    if (loc) {
#pragma unroll
        for (int a = 0; a < 3; ++a) loc[a * n + p] = u[a];
    }
}

// ---------------------------------------------------------------------------
// Active nodes (the union of the in-range corners of every occupied cell) and
// per-cell [start, end) ranges in sorted order.
// ---------------------------------------------------------------------------
static __global__ void k_cell_ranges(const unsigned* __restrict__ skeys, long long n, Geom g, unsigned* __restrict__ state,
                              unsigned* __restrict__ cstart, unsigned* __restrict__ cend,
                              const unsigned* __restrict__ perm, const uint16_t* __restrict__ sid) {
    long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s >= n) return;
    unsigned key = skeys[s];
    if (key >= g.key_max) return;
    if (s == 0 || skeys[s - 1] != key) {
        if (cstart) cstart[key] = (unsigned)s;
        const Geom& gs = (g.nspec > 1) ? g.tab[sid[perm[s]]] : g;
        int b[3];
        key_to_base(key, gs, b);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            long long nid = corner_node(gs, b, k);
            if (nid >= 0) atomicOr(&state[nid], 1u);
        }
    }
    if (cend && (s == n - 1 || skeys[s + 1] != key)) cend[key] = (unsigned)(s + 1);
}

// ---------------------------------------------------------------------------
// Warp-segmented inclusive sum over runs of equal keys (sorted order puts a
// cell's particles in adjacent lanes); the run's last lane ends with the total.
// ---------------------------------------------------------------------------
struct Runs {
    int lane, head_lane, maxrun;
    bool tail;
    __device__ __forceinline__ void init(unsigned key) {
        lane = threadIdx.x & 31;
        unsigned kp = __shfl_up_sync(FULL_MASK, key, 1);
        unsigned kn = __shfl_down_sync(FULL_MASK, key, 1);
        bool head = (lane == 0) || (kp != key);
        tail = (lane == 31) || (kn != key);
        unsigned hm = __ballot_sync(FULL_MASK, head);
        head_lane = 31 - __clz(hm & (0xffffffffu >> (31 - lane)));
        maxrun = __reduce_max_sync(FULL_MASK, (unsigned)(lane - head_lane + 1));
    }
    template <typename T>
    __device__ __forceinline__ T sum(T v) const {
        for (int off = 1; off < maxrun; off <<= 1) {
            T o = __shfl_up_sync(FULL_MASK, v, off);
            if (lane - off >= head_lane) v += o;
        }
        return v;
    }
};

// Bases of particle p: FP64 form from the position, FP32 form from the
// cell-local coordinate the previous step stored (no FP64 instructions).
template <typename T>
__device__ __forceinline__ void particle_bases(const PView<T>& P, const Geom& g, long long p, const int b[3],
                                               Bases<T>& B) {
    const long long np = P.n;
    if constexpr (sizeof(T) == 4) {
        const float u[3] = {P.loc[p], P.loc[np + p], P.loc[2 * np + p]};
        B.init_local(g, u);
    } else {
        const double x[3] = {P.pos[p], P.pos[np + p], P.pos[2 * np + p]};
        B.init(g, x, b);
    }
}

// Prefetch into L2 the bytes of elements [p0, p0 + cnt) of an array of n
// ES-byte elements (a bulk prefetch, trimmed to 16-byte boundaries inside
// the array; a hint with no effect on results).
__device__ __forceinline__ void prefetch_l2(const void* base, int es, long long n, long long p0, int cnt) {
    if (!base) return;
    const unsigned long long lo = (unsigned long long)base, hi = lo + (unsigned long long)n * es;
    unsigned long long a = lo + (unsigned long long)p0 * es;
    unsigned long long b = lo + (unsigned long long)min((long long)n, p0 + cnt) * es;
    a = max(a & ~15ULL, (lo + 15) & ~15ULL);
    b = min((b + 15) & ~15ULL, hi & ~15ULL);
    if (b > a)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"((unsigned)(b - a)) : "memory");
}

// ---------------------------------------------------------------------------
// P2G (M2G, …MPLocks.cpp:48-89): per particle and corner, mass N m, momentum
// N (m v), force -V (grad N . sigma) + N f_ext (Voigt order xx yy zz xy yz zx,
// :79-84), and (with_mg) the mass gradient grad N m of the contact path
// (…_Contact.cpp:131).  One thread per sorted slot.
//   REDUCE = 1: a cell's particles sit in adjacent lanes; their contributions
//               are summed across the lanes of the run first, then one atomic
//               per (node, field) per run.
//   REDUCE = 0: one atomic per (particle, node, field); the adds happen in L2.
// The choice (and the block size) is made per form by the autotuner.
// ---------------------------------------------------------------------------
template <typename T, int REDUCE>
__global__ void __launch_bounds__(512) k_p2g(PView<T> P, NView<T> nd, Geom g, const unsigned* __restrict__ skeys,
                                             const unsigned* __restrict__ perm, long long n, int with_mg,
                                             int mark_active) {
    long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    unsigned key = (s < n) ? skeys[s] : 0xffffffffu;
    const bool valid = key < g.key_max;
    Runs run;
    if (REDUCE) run.init(key);
    else if (!valid) return;
    const long long np = P.n, nn = nd.nn;
    int b[3] = {0, 0, 0};
    Bases<T> B;
    T m = 0, vs[6] = {0, 0, 0, 0, 0, 0}, mv[3] = {0, 0, 0}, fe[3] = {0, 0, 0};
    const Geom* gsp = &g;
    if (valid) {
        long long p = perm[s];
        gsp = &spec_geom(g, P.sid, p);
        key_to_base(key, *gsp, b);
        particle_bases<T>(P, *gsp, p, b, B);
        m = P.mass[p];
        const T V = P.vol[p];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            mv[c] = m * P.vel[c * np + p];
            fe[c] = P.fext[c * np + p];
        }
#pragma unroll
        for (int c = 0; c < 6; ++c) vs[c] = -V * P.stress[c * np + p];  // -V sigma
    }
#pragma unroll 1
    for (int k = 0; k < 8; ++k) {
        T N = 0, G[3] = {0, 0, 0};
        if (valid) B.corner(k, N, G);
        T c[10];
        c[0] = N * m;
        c[1] = N * mv[0];
        c[2] = N * mv[1];
        c[3] = N * mv[2];
        c[4] = G[0] * vs[0] + G[1] * vs[3] + G[2] * vs[5] + N * fe[0];
        c[5] = G[1] * vs[1] + G[0] * vs[3] + G[2] * vs[4] + N * fe[1];
        c[6] = G[2] * vs[2] + G[0] * vs[5] + G[1] * vs[4] + N * fe[2];
        c[7] = G[0] * m;
        c[8] = G[1] * m;
        c[9] = G[2] * m;
        const int nf = with_mg ? 10 : 7;
        if (REDUCE) {
#pragma unroll
            for (int f = 0; f < 7; ++f) c[f] = run.sum(c[f]);
            if (with_mg) {
#pragma unroll
                for (int f = 7; f < 10; ++f) c[f] = run.sum(c[f]);
            }
        }
        if (valid && (!REDUCE || run.tail)) {
            long long nid = corner_node(*gsp, b, k);
            if (nid >= 0) {
                if (mark_active) atomicOr(&nd.state[nid], 1u);  // a reduction: no load to wait for
                acc_add<T>(nd.acc, nid, c[0], c[1], c[2], c[3], c[4], c[5], c[6]);
                if (nf == 10) {
                    atomicAdd(&nd.mg[nid], c[7]);
                    atomicAdd(&nd.mg[nn + nid], c[8]);
                    atomicAdd(&nd.mg[2 * nn + nid], c[9]);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// P2G, cell-centric (P2G_REDUCE = 2).  A block takes blockDim.x consecutive
// sorted slots.  Phase 1: each slot's thread stages its particle's per-axis
// bases (N and dN/du for both nodes of each axis) and transfer quantities
// (m, m v, -V sigma, f_ext) in shared memory.  Phase 2: one thread per
// (run of equal cell keys, corner) sums that corner's contributions over the
// run's particles in slot order and issues one atomic per field.  Same
// per-particle arithmetic as k_p2g; the cross-lane shuffles of REDUCE = 1
// become shared-memory reads, and the atomics are issued by full warps.
// Shared memory: (12 + 13) values per slot (the 12 base rows padded to an odd
// stride) plus each slot's cell nodes and key, and the run starts
// (p2g_cells_smem); phase 2 takes the run's nodes from its first slot.
// ---------------------------------------------------------------------------
// Runs of equal cell keys among the block's first nslots slots (keys staged
// in shared memory, a __syncthreads after the staging): run r covers slots
// run_start[r] .. run_start[r + 1] - 1.  Returns the run count.  The slots
// need not be sorted (a cell met twice is two runs) and slots whose key is out
// of range form runs of their own, which the callers skip.
__device__ __forceinline__ int block_runs(const unsigned* skey, int nslots, int* run_start, int* wsum) {
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const bool head = t < nslots && (t == 0 || skey[t - 1] != skey[t]);
    const unsigned bal = __ballot_sync(FULL_MASK, head);
    if (lane == 0) wsum[w] = __popc(bal);
    __syncthreads();
    if (t < 32) {
        const int nw = blockDim.x >> 5;
        int v = (t < nw) ? wsum[t] : 0;
        int incl = v;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            int o = __shfl_up_sync(FULL_MASK, incl, off);
            if (t >= off) incl += o;
        }
        if (t < nw) wsum[t] = incl - v;
        if (t == 31) wsum[32] = incl;
    }
    __syncthreads();
    if (head) run_start[wsum[w] + __popc(bal & ((1u << lane) - 1u))] = t;
    const int R = wsum[32];
    if (t == 0) run_start[R] = nslots;
    __syncthreads();
    return R;
}

// Per slot, beside the values: the cell's nodes (n0, sz, sy, mask: 24 bytes)
// and the key; then the run starts (bs + 1) and the warp counts.
constexpr size_t CELL_SLOT_BYTES = 28;

// FP32 cell-run value rows: slot s is stored at row position s ^ ((s >> 3) & 7),
// a permutation inside each aligned group of 8 slots (block sizes are multiples
// of 8).  The cell runs one warp sums start 8 slots apart when cells hold 8
// particles, so in slot order their 16-byte values fall in the same four banks
// and a quarter-warp's two runs conflict; swizzled, eight consecutive runs read
// eight distinct bank groups.  Sums still run in slot order.
__device__ __forceinline__ int slot_swz(int s) { return s ^ ((s >> 3) & 7); }

template <typename T>
__host__ __device__ constexpr size_t p2g_cells_smem(int bs) {
    return (sizeof(T) == 4 ? (size_t)25 * bs * 4 : ((size_t)12 * (bs + 1) + (size_t)13 * bs) * sizeof(T)) +
           (size_t)bs * CELL_SLOT_BYTES + (size_t)(bs + 1) * 4 + 64 * 4;
}

// The slot arrays that follow the values (8-byte aligned: even bs).
struct CellSlots {
    long long *n0, *sz;
    int* sy;
    unsigned *mask, *key;
    int *run_start, *wsum;
    __device__ __forceinline__ CellSlots(unsigned char* at, int bs) {
        n0 = reinterpret_cast<long long*>(at);
        sz = n0 + bs;
        sy = reinterpret_cast<int*>(sz + bs);
        mask = reinterpret_cast<unsigned*>(sy + bs);
        key = mask + bs;
        run_start = reinterpret_cast<int*>(key + bs);  // bs + 1
        wsum = run_start + bs + 1;                     // 32 warp counts + total
    }
    __device__ __forceinline__ void put(int t, const CellNodes& c) const {
        n0[t] = c.n0;
        sz[t] = c.sz;
        sy[t] = c.sy;
        mask[t] = c.mask;
    }
    // corner k's node of the cell staged at slot a, or -1 out of range
    __device__ __forceinline__ long long node(int a, int k) const {
        if (!((mask[a] >> k) & 1u)) return -1;
        CellNodes c;
        c.n0 = n0[a];
        c.sz = sz[a];
        c.sy = sy[a];
        return cell_node(c, k);
    }
};

// CPT corners per phase-2 thread (1, 2 or 4): the corners sharing the
// thread's x (CPT 4) or x and y (CPT 2) bases, so a particle's quantities are
// read from shared memory 8 / CPT times instead of 8.  BS, the block size, is
// a compile-time constant so the shared-memory rows sit at fixed offsets from
// one address.
// A cell-run P2G block of BS slots in shared memory: the per-axis bases, the
// transfer quantities (m, m v (3), -V sigma (6), f_ext (3)) and the slots
// (cell nodes, key, runs).  FP64: 12 rows of BS + 1 bases (the odd stride puts
// the two nodes' values of an axis in different banks; Nx0 Nx1 Ny0 Ny1 Nz0
// Nz1 gx0 gx1 gy0 gy1 gz0 gz1) and 13 rows of BS quantities.  FP32: six rows
// of BS float4 ({Nx0 Nx1 gx0 gx1}, y, z, {m, m v}, {-V sigma 0..3},
// {-V sigma 4..5, f_ext 0..1}) and a row of f_ext 2, so a scatter thread reads
// a particle with seven shared loads.
template <typename T, int BS>
struct P2GBlock {
    static constexpr int S = BS + 1;
    T* sw;
    T* sq;
    CellSlots cs;
    __device__ __forceinline__ explicit P2GBlock(unsigned char* raw)
        : sw(reinterpret_cast<T*>(raw)), sq(sw + (sizeof(T) == 4 ? 24 * BS : 12 * S)),
          cs(reinterpret_cast<unsigned char*>(sq + (sizeof(T) == 4 ? BS : 13 * BS)), BS) {}

    // slot t's particle: bases, mass m, volume V, velocity v, external force fe, stress sig, its cell's nodes
    __device__ __forceinline__ void stage(int t, const Bases<T>& B, T m, T V, const T v[3], const T fe[3],
                                          const T sig[6], const CellNodes& cn) const {
        if constexpr (sizeof(T) == 4) {
            static_assert(BS % 8 == 0, "slot swizzle groups");
            float4* sv = reinterpret_cast<float4*>(sw);
            const int u = slot_swz(t);
            sv[u] = make_float4(B.Nx[0], B.Nx[1], B.gx[0], B.gx[1]);
            sv[BS + u] = make_float4(B.Ny[0], B.Ny[1], B.gy[0], B.gy[1]);
            sv[2 * BS + u] = make_float4(B.Nz[0], B.Nz[1], B.gz[0], B.gz[1]);
            sv[3 * BS + u] = make_float4(m, m * v[0], m * v[1], m * v[2]);
            sv[4 * BS + u] = make_float4(-V * sig[0], -V * sig[1], -V * sig[2], -V * sig[3]);
            sv[5 * BS + u] = make_float4(-V * sig[4], -V * sig[5], fe[0], fe[1]);
            sq[u] = fe[2];
            cs.put(t, cn);
            return;
        }
        sw[0 * S + t] = B.Nx[0];
        sw[1 * S + t] = B.Nx[1];
        sw[2 * S + t] = B.Ny[0];
        sw[3 * S + t] = B.Ny[1];
        sw[4 * S + t] = B.Nz[0];
        sw[5 * S + t] = B.Nz[1];
        sw[6 * S + t] = B.gx[0];
        sw[7 * S + t] = B.gx[1];
        sw[8 * S + t] = B.gy[0];
        sw[9 * S + t] = B.gy[1];
        sw[10 * S + t] = B.gz[0];
        sw[11 * S + t] = B.gz[1];
        sq[t] = m;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            sq[(1 + c) * BS + t] = m * v[c];
            sq[(10 + c) * BS + t] = fe[c];
        }
#pragma unroll
        for (int c = 0; c < 6; ++c) sq[(4 + c) * BS + t] = -V * sig[c];
        cs.put(t, cn);
    }

    // After the staging and a __syncthreads (keys in cs.key for the first nslots
    // slots, out of range where nothing was staged): one thread per (cell run,
    // CPT corners) sums the run's contributions in slot order and issues one
    // atomic per field; mark_active also marks the corners active.  MG: also the
    // node mass gradients.
    //
    // FP32: a warp holds consecutive runs, the TPR threads of a run in
    // adjacent lanes.  When run r's cell follows run r - 1's in x (key + 1),
    // the x = 1 corners of r - 1 are the x = 0 corners of r: one shuffle of
    // the sums, TPR / 2 lanes up, adds them to r's, and only r's lanes issue
    // the atomics (in the batch about three runs in four have such a
    // neighbour, so a third of the corner atomics go).
    template <int CPT, bool MG>
    __device__ __forceinline__ void scatter(const NView<T>& nd, const Geom& g, int nslots, int mark_active) const {
        static_assert(CPT == 1 || CPT == 2 || CPT == 4, "corners per thread");
        constexpr int bs = BS;
        const int t = threadIdx.x, lane = t & 31;
        const long long nn = nd.nn;
        const unsigned* skey = cs.key;
        const int R = block_runs(skey, nslots, cs.run_start, cs.wsum);
        constexpr int TPR = 8 / CPT;  // threads per run
        const int nitems = R * TPR;
        // whole warps take the loop together (the merge shuffles)
        for (int item = t; item - lane < nitems; item += bs) {
            const bool live = item < nitems;
            const int r = live ? item / TPR : 0, kq = item % TPR, k0 = kq * CPT;  // corners k0 .. k0 + CPT - 1
            const int a = cs.run_start[r];
            // slots outside the grid (and lanes past the items) sum nothing
            const bool inb = live && skey[a] < g.key_max;
            const int e = inb ? cs.run_start[r + 1] : a;
            T am[CPT], ap0[CPT], ap1[CPT], ap2[CPT], af0[CPT], af1[CPT], af2[CPT], g0[CPT], g1[CPT], g2[CPT];
    #pragma unroll
            for (int j = 0; j < CPT; ++j) am[j] = ap0[j] = ap1[j] = ap2[j] = af0[j] = af1[j] = af2[j] = g0[j] = g1[j] = g2[j] = 0;
            for (int i = a; i < e; ++i) {
                T m, mv0, mv1, mv2, v0, v1, v2, v3, v4, v5, fe0, fe1, fe2;
                float4 X, Y, Z;
                if constexpr (sizeof(T) == 4) {
                    const float4* sv = reinterpret_cast<const float4*>(sw);
                    const int u = slot_swz(i);
                    X = sv[u];
                    Y = sv[BS + u];
                    Z = sv[2 * BS + u];
                    const float4 q0 = sv[3 * BS + u], q1 = sv[4 * BS + u], q2 = sv[5 * BS + u];
                    m = q0.x, mv0 = q0.y, mv1 = q0.z, mv2 = q0.w;
                    v0 = q1.x, v1 = q1.y, v2 = q1.z, v3 = q1.w;
                    v4 = q2.x, v5 = q2.y, fe0 = q2.z, fe1 = q2.w;
                    fe2 = sq[u];
                } else {
                    m = sq[i], mv0 = sq[1 * bs + i], mv1 = sq[2 * bs + i], mv2 = sq[3 * bs + i];
                    v0 = sq[4 * bs + i], v1 = sq[5 * bs + i], v2 = sq[6 * bs + i];
                    v3 = sq[7 * bs + i], v4 = sq[8 * bs + i], v5 = sq[9 * bs + i];
                    fe0 = sq[10 * bs + i], fe1 = sq[11 * bs + i], fe2 = sq[12 * bs + i];
                }
                if constexpr (sizeof(T) == 4 && CPT >= 2) {
                    // FP32, corners sharing x (and y) bases: the products are
                    // regrouped around the z factor.  With A = Nx Ny, Bx = Ny gx,
                    // By = Nx gy a corner's N = A Nz, G = -(Bx Nz, By Nz, A gz),
                    // so its seven sums are N m, N m v and Nz c + gz d, with
                    // c and d formed once per slot and (x, y) pair.
                    const int ix = (k0 >> 2) & 1;
                    const float nx = ix ? X.y : X.x, gxv = ix ? X.w : X.z;
#pragma unroll
                    for (int jy = 0; jy < CPT / 2; ++jy) {
                        const int iy = CPT == 4 ? jy : ((k0 >> 1) & 1);
                        const float ny = iy ? Y.y : Y.x, gyv = iy ? Y.w : Y.z;
                        const float A = nx * ny, Bx = ny * gxv, By = nx * gyv;
                        const float Am = A * m, Am0 = A * mv0, Am1 = A * mv1, Am2 = A * mv2;
                        const float c0 = A * fe0 - Bx * v0 - By * v3;
                        const float c1 = A * fe1 - By * v1 - Bx * v3;
                        const float c2 = A * fe2 - Bx * v5 - By * v4;
                        const float d0 = -A * v5, d1 = -A * v4, d2 = -A * v2;
#pragma unroll
                        for (int iz = 0; iz < 2; ++iz) {
                            const int j = 2 * jy + iz;
                            const float nz = iz ? Z.y : Z.x, gzv = iz ? Z.w : Z.z;
                            am[j] += nz * Am;
                            ap0[j] += nz * Am0;
                            ap1[j] += nz * Am1;
                            ap2[j] += nz * Am2;
                            af0[j] = fmaf(gzv, d0, fmaf(nz, c0, af0[j]));
                            af1[j] = fmaf(gzv, d1, fmaf(nz, c1, af1[j]));
                            af2[j] = fmaf(gzv, d2, fmaf(nz, c2, af2[j]));
                            if constexpr (MG) {
                                g0[j] -= nz * (Bx * m);
                                g1[j] -= nz * (By * m);
                                g2[j] -= gzv * Am;
                            }
                        }
                    }
                    continue;
                }
    #pragma unroll
                for (int j = 0; j < CPT; ++j) {
                    const int k = k0 + j;
                    const int ix = (k >> 2) & 1, iy = (k >> 1) & 1, iz = k & 1;
                    T nx, ny, nz, gxv, gyv, gzv;
                    if constexpr (sizeof(T) == 4) {
                        nx = ix ? X.y : X.x, gxv = ix ? X.w : X.z;
                        ny = iy ? Y.y : Y.x, gyv = iy ? Y.w : Y.z;
                        nz = iz ? Z.y : Z.x, gzv = iz ? Z.w : Z.z;
                    } else {
                        nx = sw[ix * S + i], ny = sw[(2 + iy) * S + i], nz = sw[(4 + iz) * S + i];
                        gxv = sw[(6 + ix) * S + i], gyv = sw[(8 + iy) * S + i], gzv = sw[(10 + iz) * S + i];
                    }
                    const T N = nx * ny * nz;
                    const T G0 = -(ny * nz) * gxv;
                    const T G1 = -(nx * nz) * gyv;
                    const T G2 = -(nx * ny) * gzv;
                    am[j] += N * m;
                    ap0[j] += N * mv0;
                    ap1[j] += N * mv1;
                    ap2[j] += N * mv2;
                    af0[j] += G0 * v0 + G1 * v3 + G2 * v5 + N * fe0;
                    af1[j] += G1 * v1 + G0 * v3 + G2 * v4 + N * fe1;
                    af2[j] += G2 * v2 + G0 * v5 + G1 * v4 + N * fe2;
                    if constexpr (MG) {
                        g0[j] += G0 * m;
                        g1[j] += G1 * m;
                        g2[j] += G2 * m;
                    }
                }
            }
            bool skip = !inb;
            if constexpr (sizeof(T) == 4) {
                constexpr int SH = TPR / 2;  // lanes from run r - 1's x = 1 corners to run r's x = 0 corners
                const bool recv = inb && kq < SH && lane >= SH && r > 0 && skey[cs.run_start[r - 1]] + 1u == skey[a];
#pragma unroll
                for (int j = 0; j < CPT; ++j) {
                    const float x0 = __shfl_up_sync(FULL_MASK, am[j], SH), x1 = __shfl_up_sync(FULL_MASK, ap0[j], SH);
                    const float x2 = __shfl_up_sync(FULL_MASK, ap1[j], SH), x3 = __shfl_up_sync(FULL_MASK, ap2[j], SH);
                    const float x4 = __shfl_up_sync(FULL_MASK, af0[j], SH), x5 = __shfl_up_sync(FULL_MASK, af1[j], SH);
                    const float x6 = __shfl_up_sync(FULL_MASK, af2[j], SH);
                    if (recv) {
                        am[j] += x0, ap0[j] += x1, ap1[j] += x2, ap2[j] += x3;
                        af0[j] += x4, af1[j] += x5, af2[j] += x6;
                    }
                    if constexpr (MG) {
                        const float y0 = __shfl_up_sync(FULL_MASK, g0[j], SH);
                        const float y1 = __shfl_up_sync(FULL_MASK, g1[j], SH);
                        const float y2 = __shfl_up_sync(FULL_MASK, g2[j], SH);
                        if (recv) g0[j] += y0, g1[j] += y1, g2[j] += y2;
                    }
                }
                // a sender's sums went to the lane SH up (lanes near the warp's top read their own false)
                if (__shfl_down_sync(FULL_MASK, recv ? 1 : 0, SH) && kq >= SH) skip = true;
            }
            if (skip) continue;
#pragma unroll
            for (int j = 0; j < CPT; ++j) {
                const long long nid = cs.node(a, k0 + j);
                if (nid < 0) continue;
                // active nodes: the in-range corners of occupied cells (b_Active, …MPLocks.cpp:36)
                if (mark_active) atomicOr(&nd.state[nid], 1u);  // a reduction: no load to wait for
                acc_add<T>(nd.acc, nid, am[j], ap0[j], ap1[j], ap2[j], af0[j], af1[j], af2[j]);
                if constexpr (MG) {
                    atomicAdd(&nd.mg[nid], g0[j]);
                    atomicAdd(&nd.mg[nn + nid], g1[j]);
                    atomicAdd(&nd.mg[2 * nn + nid], g2[j]);
                }
            }
        }
    }
};

// MG: also the contact path's node mass gradients (output steps only).
template <typename T, int CPT, int BS, bool MG>
__device__ __forceinline__ void p2g_cells_run(const PView<T>& P, const NView<T>& nd, const Geom& g,
                                              const unsigned* __restrict__ skeys, const unsigned* __restrict__ perm,
                                              long long n, int mark_active) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const P2GBlock<T, BS> blk(smem_raw);
    const int t = threadIdx.x;
    const long long s = blockIdx.x * (long long)BS + t;
    const unsigned key = (s < n) ? skeys[s] : 0xffffffffu;
    const long long np = P.n;
    if (key < g.key_max) {
        const long long p = perm ? perm[s] : s;
        const Geom& gs = spec_geom(g, P.sid, p);
        int b[3];
        key_to_base(key, gs, b);
        Bases<T> B;
        particle_bases<T>(P, gs, p, b, B);
        T v[3], fe[3], sig[6];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            v[c] = P.vel[c * np + p];
            fe[c] = P.fext[c * np + p];
        }
#pragma unroll
        for (int c = 0; c < 6; ++c) sig[c] = P.stress[c * np + p];
        blk.stage(t, B, P.mass[p], P.vol[p], v, fe, sig, cell_nodes(gs, b));
    }
    blk.cs.key[t] = key;
    __syncthreads();
    blk.template scatter<CPT, MG>(nd, g, (int)min((long long)BS, n - blockIdx.x * (long long)BS), mark_active);
}

// FP32 with 1 or 2 corners per thread: registers capped for 1536 resident
// threads per SM (40 registers, no spills at 2 corners), which hides more of
// the staging loads' latency than 48 registers at 1280 threads.
template <typename T, int CPT>
__host__ __device__ constexpr int cells_min_blocks(int bs) {
    return sizeof(T) == 4 && CPT < 4 ? 1536 / bs : 1;
}

template <typename T, int CPT, int BS>
__global__ void __launch_bounds__(BS, cells_min_blocks<T, CPT>(BS)) k_p2g_cells(PView<T> P, NView<T> nd, Geom g, const unsigned* __restrict__ skeys,
                                                   const unsigned* __restrict__ perm, long long n, int mark_active) {
    p2g_cells_run<T, CPT, BS, false>(P, nd, g, skeys, perm, n, mark_active);
}

template <typename T, int CPT, int BS>
__global__ void __launch_bounds__(BS) k_p2g_cells_mg(PView<T> P, NView<T> nd, Geom g,
                                                      const unsigned* __restrict__ skeys,
                                                      const unsigned* __restrict__ perm, long long n, int mark_active) {
    p2g_cells_run<T, CPT, BS, true>(P, nd, g, skeys, perm, n, mark_active);
}

// ---------------------------------------------------------------------------
// Displacement control (…MPLocks.cpp:143-174; contact :283-297, :416-432).
// The reference overwrites node velocity/momentum/force from each controlled
// particle in list order, so a node shared by several keeps the last one's.
// k_dc_claim records, per node and axis, the largest list position writing
// it, and marks the node (NODE_CLAIMED in its state word) so the node phases
// read the claims of marked nodes only; node_dc lets only the claiming
// particle write.  contact: every particle claims all three axes, so the axis-0
// claim word stands for the three (one atomic per corner instead of three).
// ---------------------------------------------------------------------------
static __global__ void k_dc_claim(const unsigned* __restrict__ dclist, int ndc, const unsigned* __restrict__ keys,
                           const uint8_t* __restrict__ pflags, Geom g, unsigned* __restrict__ owner, long long nn,
                           int contact, const uint16_t* __restrict__ sid, unsigned* __restrict__ state) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ndc) return;
    unsigned p = dclist[k];
    unsigned key = keys[p];
    if (key >= g.key_max) return;
    const Geom& gs = spec_geom(g, sid, p);
    unsigned axes = contact ? 7u : (pflags[p] & 7u);
    int b[3];
    key_to_base(key, gs, b);
    for (int c8 = 0; c8 < 8; ++c8) {
        long long nid = corner_node(gs, b, c8);
        if (nid < 0) continue;
        for (int a = 0; a < 3; ++a)
            if ((axes & (1u << a)) && !(contact && a > 0)) atomicMax(&owner[a * nn + nid], (unsigned)k + 1u);
        if (axes) atomicOr(&state[nid], NODE_CLAIMED);
    }
}

// ---------------------------------------------------------------------------
// Grid momentum update with boundary conditions (IntegrateGrid,
// …MPLocks.cpp:90-142).  Non-contact order: damping, x-wall Coulomb friction
// on y (:106-124), zero fixed axes (y-fixed nodes accumulate the reaction
// force, :129), then p += f dt.  Contact order (…_Contact.cpp:250-276):
// damping, p += f dt, then zero fixed axes; optionally Coulomb friction on
// the x/y tangents of z-fixed nodes (floor_friction, an extension).
// Damping is skipped when its coefficient is zero (f - 0*x == f).
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void coulomb(T p_t, T& f_t, T fn, T mu, T dt) {
    T trial = p_t + f_t * dt;
    T ff = mu * (T)((T(0) < -trial) - (-trial < T(0))) * fabs(fn);
    if (fabs(ff * dt) > fabs(trial)) ff *= fabs(trial / dt) / fabs(ff);
    f_t += ff;
}

// The update of one node's momentum p and force f in registers; zero[c]: the
// axis is fixed (its velocity is zeroed too); ft_y: the y reaction force of a
// y-fixed node.  friction is read only where a friction law applies.
template <typename T>
__device__ __forceinline__ void grid_update_regs(const NView<T>& nd, long long i, unsigned fx, T p[3], T f[3], T dt,
                                                 double damping, int contact, int floor_friction, bool zero[3],
                                                 T& ft_y, T dfr[3]) {
    dfr[0] = dfr[1] = dfr[2] = (T)0;  // the force each friction law added (for the friction work)
    if (damping != 0.0) {
        T pp = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
        if (sqrt(pp) > (T)1.0e-24) {
            T inv = (T)1 / sqrt(pp);
            T nrm[3] = {p[0] * inv, p[1] * inv, p[2] * inv};
            T sc = (T)damping * fabs(f[0] * nrm[0] + f[1] * nrm[1] + f[2] * nrm[2]);
#pragma unroll
            for (int c = 0; c < 3; ++c) f[c] = f[c] - sc * nrm[c];
        }
    }
    zero[0] = zero[1] = zero[2] = false;
    ft_y = 0;
    if (!contact) {
        if (fx & 1u) {
            T trial_y = p[1] + f[1] * dt;
            if (fabs(trial_y * dt) > (T)1.0e-24 && f[0] > (T)0) {
                const T f0 = f[1];
                coulomb<T>(p[1], f[1], f[0], (T)nd.friction[i], dt);
                dfr[1] = f[1] - f0;
            }
            zero[0] = true;
            p[0] = 0;
            f[0] = 0;
        }
        if (fx & 2u) {
            ft_y = f[1];
            zero[1] = true;
            p[1] = 0;
            f[1] = 0;
        }
        if (fx & 4u) {
            zero[2] = true;
            p[2] = 0;
            f[2] = 0;
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) p[c] = p[c] + f[c] * dt;
    } else {
        if (floor_friction && (fx & 4u) && nd.friction[i] > 0.0 && f[2] < (T)0) {
            T fz = f[2], mu = (T)nd.friction[i];
#pragma unroll
            for (int t = 0; t < 2; ++t) {
                T trial = p[t] + f[t] * dt;
                if (fabs(trial * dt) > (T)1.0e-24) {
                    const T f0 = f[t];
                    coulomb<T>(p[t], f[t], fz, mu, dt);
                    dfr[t] = f[t] - f0;
                }
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) p[c] = p[c] + f[c] * dt;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (fx & (1u << c)) {
                if (c == 1) ft_y = f[1];
                zero[c] = true;
                p[c] = 0;
                f[c] = 0;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// G2P pass 1 (…MPLocks.cpp:489-510): v_p += N (f_i/m_i) dt over the corners
// in findAdjacentGridPoints order, fused with the velocity remap (:539-564):
// each particle then scatters N m_p v_p, summed per run before the atomic.
// Contact path: particles flagged b_DisplacementControl are skipped.
// ---------------------------------------------------------------------------
template <typename T, int BATCH>
__global__ void __launch_bounds__(256) k_pass1_remap(PView<T> P, NView<T> nd, Geom g,
                                                     const unsigned* __restrict__ skeys,
                                                     const unsigned* __restrict__ perm, long long n, T dt,
                                                     T mass_min, int contact) {
    long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    unsigned key = (s < n) ? skeys[s] : 0xffffffffu;
    Runs run;
    run.init(key);
    // key_ok: the run has grid nodes (its tail lane issues the atomics even
    // when its own particle is skipped); valid: this particle takes part
    const bool key_ok = key < g.key_max;
    bool valid = key_ok;
    const long long np = P.n, nn = nd.nn;
    long long p = 0;
    const Geom* gsp = &g;
    int b[3] = {0, 0, 0};
    if (key_ok) {
        p = perm[s];
        if (contact && (P.pflags[p] & 8u)) valid = false;
        gsp = &spec_geom(g, P.sid, p);
        key_to_base(key, *gsp, b);
    }
    Bases<T> B;
    T m = 0, v[3] = {0, 0, 0};
    if (valid) {
        particle_bases<T>(P, *gsp, p, b, B);
        m = P.mass[p];
#pragma unroll
        for (int c = 0; c < 3; ++c) v[c] = P.vel[c * np + p];
        // BATCH: every corner's record is requested before any is used (one
        // round trip to memory instead of eight, at more registers); the sum
        // runs in corner order either way
        if constexpr (BATCH) {
            Quad<T> r[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const long long nid = corner_node(*gsp, b, k);
                r[k] = nid >= 0 ? ld_quad(nd.rec + 8 * nid) : Quad<T>{(T)0, (T)0, (T)0, (T)0};
            }
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                if (!(r[k].w != (T)0)) continue;  // out of range or m <= mass_min
                T N, G[3];
                B.corner(k, N, G);
                v[0] = v[0] + N * r[k].x * dt;
                v[1] = v[1] + N * r[k].y * dt;
                v[2] = v[2] + N * r[k].z * dt;
            }
        } else {
#pragma unroll 1
            for (int k = 0; k < 8; ++k) {
                const long long nid = corner_node(*gsp, b, k);
                if (nid < 0) continue;
                const Quad<T> r = ld_quad(nd.rec + 8 * nid);
                if (!(r.w != (T)0)) continue;
                T N, G[3];
                B.corner(k, N, G);
                v[0] = v[0] + N * r.x * dt;
                v[1] = v[1] + N * r.y * dt;
                v[2] = v[2] + N * r.z * dt;
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) P.vel[c * np + p] = v[c];
    }
    T mv[3] = {m * v[0], m * v[1], m * v[2]};
#pragma unroll 1
    for (int k = 0; k < 8; ++k) {
        T N = 0, G[3];
        if (valid) B.corner(k, N, G);
        T q0 = run.sum(N * mv[0]);
        T q1 = run.sum(N * mv[1]);
        T q2 = run.sum(N * mv[2]);
        if (key_ok && run.tail) {
            long long nid = corner_node(*gsp, b, k);
            if (nid >= 0) {
                q_add<T>(nd.q, nid, q0, q1, q2);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// G2P pass 1 + velocity remap, cell-centric (used with P2G mode 2): each slot's
// thread updates its particle's velocity from the node records (in corner
// order, as k_pass1_remap) and stages N (per axis) and m v in shared memory;
// one thread per (cell run, corner) then sums N m v over the run in slot order
// and issues three atomics.  Skipped particles (platen on the contact path)
// stay in their run with zero weight.
// ---------------------------------------------------------------------------
template <typename T>
__host__ __device__ constexpr size_t pass1_cells_smem(int bs) {
    return (sizeof(T) == 4 ? (size_t)9 * bs * 4 : ((size_t)6 * (bs + 1) + (size_t)3 * bs) * sizeof(T)) +
           (size_t)bs * CELL_SLOT_BYTES + (size_t)(bs + 1) * 4 + 64 * 4;
}

// FP32 with 1 or 2 corners per thread: registers capped for 1536 resident
// threads per SM (40 registers, a few bytes spilled), about 10% faster than
// 56 registers at 1152 threads: the kernel waits on its record gathers, and
// more resident warps keep more of them in flight.
template <typename T, int CPT, int BS>
__global__ void __launch_bounds__(BS, cells_min_blocks<T, CPT>(BS)) k_pass1_cells(PView<T> P, NView<T> nd, Geom g,
                                                     const unsigned* __restrict__ skeys,
                                                     const unsigned* __restrict__ perm, long long n, T dt,
                                                     T mass_min, int contact) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int bs = BS;
    const int t = threadIdx.x;
    // FP64: 6 rows of S = bs + 1 (odd stride: the two nodes' values of an axis
    // in different banks) Nx0 Nx1 Ny0 Ny1 Nz0 Nz1, then 3 rows of bs m v.
    // FP32: two rows of bs float4 {Nx0 Nx1 Ny0 Ny1} {Nz0 Nz1 mv0 mv1} and a row of mv2.
    constexpr int S = bs + 1;
    constexpr bool F32 = sizeof(T) == 4;
    T* sn = reinterpret_cast<T*>(smem_raw);
    T* smv = sn + (F32 ? 8 * bs : 6 * S);
    CellSlots cs(reinterpret_cast<unsigned char*>(smv + (F32 ? bs : 3 * bs)), bs);
    unsigned* skey = cs.key;
    const long long s = blockIdx.x * (long long)bs + t;
    const unsigned key = (s < n) ? skeys[s] : 0xffffffffu;
    const bool key_ok = key < g.key_max;
    const long long np = P.n, nn = nd.nn;
    if (key_ok) {
        const long long p = perm ? perm[s] : s;
        const Geom& gs = spec_geom(g, P.sid, p);
        int b[3];
        key_to_base(key, gs, b);
        const CellNodes cn = cell_nodes(gs, b);
        cs.put(t, cn);
        const bool valid = !(contact && (P.pflags[p] & 8u));
        T N6[6] = {0, 0, 0, 0, 0, 0}, mv[3] = {0, 0, 0};
        if (valid) {
            Bases<T> B;
            particle_bases<T>(P, gs, p, b, B);
            const T m = P.mass[p];
            T v[3] = {P.vel[p], P.vel[np + p], P.vel[2 * np + p]};
            // four corners' records requested before any is used; summed in corner order
#pragma unroll(F32 ? 2 : 1)
            for (int h = 0; h < 2; ++h) {
                Quad<T> rq[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int k = 4 * h + j;
                    const Quad<T> z{(T)0, (T)0, (T)0, (T)0};
                    rq[j] = ((cn.mask >> k) & 1u) ? ld_quad(nd.rec + 8 * cell_node(cn, k)) : z;
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (!(rq[j].w != (T)0)) continue;
                    T N, G[3];
                    B.corner(4 * h + j, N, G);
                    v[0] = v[0] + N * rq[j].x * dt;
                    v[1] = v[1] + N * rq[j].y * dt;
                    v[2] = v[2] + N * rq[j].z * dt;
                }
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                P.vel[c * np + p] = v[c];
                mv[c] = m * v[c];
            }
            N6[0] = B.Nx[0];
            N6[1] = B.Nx[1];
            N6[2] = B.Ny[0];
            N6[3] = B.Ny[1];
            N6[4] = B.Nz[0];
            N6[5] = B.Nz[1];
        }
        if constexpr (F32) {
            static_assert(BS % 8 == 0, "slot swizzle groups");
            float4* sv = reinterpret_cast<float4*>(sn);
            const int u = slot_swz(t);
            sv[u] = make_float4(N6[0], N6[1], N6[2], N6[3]);
            sv[bs + u] = make_float4(N6[4], N6[5], mv[0], mv[1]);
            smv[u] = mv[2];
        } else {
#pragma unroll
            for (int c = 0; c < 6; ++c) sn[c * S + t] = N6[c];
#pragma unroll
            for (int c = 0; c < 3; ++c) smv[c * bs + t] = mv[c];
        }
    }
    skey[t] = key;
    __syncthreads();
    const int R = block_runs(skey, (int)min((long long)bs, n - blockIdx.x * (long long)bs), cs.run_start, cs.wsum);
    constexpr int TPR = 8 / CPT;  // threads per run; each sums CPT corners sharing its x (and y) bases
    for (int item = t; item < R * TPR; item += bs) {
        const int r = item / TPR, k0 = (item % TPR) * CPT;
        const int a = cs.run_start[r], e = cs.run_start[r + 1];
        if (!(skey[a] < g.key_max)) continue;  // slots outside the grid
        T q0[CPT], q1[CPT], q2[CPT];
#pragma unroll
        for (int j = 0; j < CPT; ++j) q0[j] = q1[j] = q2[j] = 0;
        for (int i = a; i < e; ++i) {
            T mv0, mv1, mv2;
            float4 A, B;
            if constexpr (F32) {
                const float4* sv = reinterpret_cast<const float4*>(sn);
                const int u = slot_swz(i);
                A = sv[u];
                B = sv[bs + u];
                mv0 = B.z, mv1 = B.w, mv2 = smv[u];
            } else {
                mv0 = smv[i], mv1 = smv[bs + i], mv2 = smv[2 * bs + i];
            }
#pragma unroll
            for (int j = 0; j < CPT; ++j) {
                const int k = k0 + j;
                const int ix = (k >> 2) & 1, iy = (k >> 1) & 1, iz = k & 1;
                T N;
                if constexpr (F32)
                    N = (ix ? A.y : A.x) * (iy ? A.w : A.z) * (iz ? B.y : B.x);
                else
                    N = sn[ix * S + i] * sn[(2 + iy) * S + i] * sn[(4 + iz) * S + i];
                q0[j] += N * mv0;
                q1[j] += N * mv1;
                q2[j] += N * mv2;
            }
        }
#pragma unroll
        for (int j = 0; j < CPT; ++j) {
            const long long nid = cs.node(a, k0 + j);
            if (nid < 0) continue;
            q_add<T>(nd.q, nid, q0[j], q1[j], q2[j]);
        }
    }
}

// Displacement control from the node's side: for each axis whose last-writer
// claim (list position + 1, k_dc_claim) is set, the claiming platen particle's
// velocity v, momentum m v and zero force.
template <typename T>
__device__ __forceinline__ void node_dc_regs(const unsigned own[3], const unsigned* __restrict__ dclist,
                                             const T* __restrict__ pvel, long long np, T m, T v[3], bool vset[3],
                                             T p[3], bool fzero[3]) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (!own[a]) continue;
        const T vp = pvel[a * np + dclist[own[a] - 1]];
        v[a] = vp;
        vset[a] = true;
        p[a] = m * vp;
        fzero[a] = true;
    }
}

// The node work between P2G and pass 1, one pass over the active nodes with
// the node's values in registers: displacement control (non-contact: before
// the update, …MPLocks.cpp:143-174), the grid update (IntegrateGrid, :90-142;
// contact :242-277), displacement control (contact: after it), then the
// record (f/m, m > m_min), the divisor of G2P pass 1 (:508).  The updated
// momentum and the mass also go to the record's second half for phase B
// (which overwrites it with p/m and v); clean (not an output step): the
// node's mass, momentum and force are zeroed here, for the next step's P2G.
//
// work (when given): the step's boundary work in FP64, added to work[0]
// (displacement control) and work[1] (friction).  No counterpart in the
// reference, whose energy report has no external-work term
// (PhysicsEngine.cpp:140-156).  A displacement-controlled node axis takes the
// platen's velocity v and its force f is zeroed (…MPLocks.cpp:143-174;
// contact …_Contact.cpp:283-297), so the platen supplies -f there; the
// velocity field pass 2 strains the particles with is v at that node, so the
// platen's work is -f v dt.  A friction law adds df to a tangent force, whose
// work is df (p/m) dt at the updated momentum.  Summed per node in the
// form's type, per thread in double, then over the warp and added once.
template <typename T>
__device__ __forceinline__ void work_add(double* work, double w_dc, double w_fr, double dt) {
    if (!work || !__any_sync(FULL_MASK, w_dc != 0.0 || w_fr != 0.0)) return;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        w_dc += __shfl_down_sync(FULL_MASK, w_dc, off);
        w_fr += __shfl_down_sync(FULL_MASK, w_fr, off);
    }
    if ((threadIdx.x & 31) == 0) {
        if (w_dc != 0.0) atomicAdd(work, w_dc * dt);
        if (w_fr != 0.0) atomicAdd(work + 1, w_fr * dt);
    }
}

template <typename T>
__device__ __forceinline__ double dc_power(const T f[3], const T v[3], const bool fz[3]) {
    T s = (T)0;
#pragma unroll
    for (int c = 0; c < 3; ++c)
        if (fz[c]) s -= f[c] * v[c];
    return fps_f2d_form(s);
}

template <typename T>
__global__ void __launch_bounds__(256, 4) k_node_phase_a(NView<T> nd, T dt, double damping, int contact, int floor_friction,
                               const unsigned* __restrict__ dclist, int ndc, const T* __restrict__ pvel, long long np,
                               T mass_min, int clean, double* work, double dtd) {
    const long long nn = nd.nn;
    double w_dc = 0.0, w_fr = 0.0;
    NODE_LOOP_AHEAD(nd, i) {
        const unsigned st = nd.state[i];
        if (!nd.alist && !(st & 1u)) continue;  // the list holds active nodes only
        const Quad<T> a0 = ld_quad(nd.acc + 8 * i), a1 = ld_quad(nd.acc + 8 * i + 4);
        const T m = a0.x;
        T p[3] = {a0.y, a0.z, a0.w}, f[3] = {a1.x, a1.y, a1.z}, v[3] = {0, 0, 0};
        const unsigned fx = nd.fixed[i];
        unsigned own[3] = {0u, 0u, 0u};
        if (ndc && (st & NODE_CLAIMED)) {
            // contact: every controlled particle claims all three axes, so one claim word serves them
#pragma unroll
            for (int a = 0; a < 3; ++a) own[a] = (contact && a > 0) ? own[0] : nd.owner[a * nn + i];
        }
        bool vset[3] = {false, false, false}, fz[3] = {false, false, false};
        if (!contact) {
            node_dc_regs<T>(own, dclist, pvel, np, m, v, vset, p, fz);
            if (work && (fz[0] | fz[1] | fz[2])) w_dc += dc_power<T>(f, v, fz);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c)
            if (fz[c]) f[c] = (T)0;
        bool zero[3];
        T ft_y, dfr[3];
        grid_update_regs<T>(nd, i, fx, p, f, dt, damping, contact, floor_friction, zero, ft_y, dfr);
        if (work && (dfr[0] != (T)0 || dfr[1] != (T)0) && m > mass_min)
            w_fr += fps_f2d_form((dfr[0] * p[0] + dfr[1] * p[1]) / m);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (zero[c]) {
                v[c] = (T)0;
                vset[c] = true;
            }
            fz[c] = false;
        }
        if (contact) {
            node_dc_regs<T>(own, dclist, pvel, np, m, v, vset, p, fz);
            if (work && (fz[0] | fz[1] | fz[2])) w_dc += dc_power<T>(f, v, fz);
#pragma unroll
            for (int c = 0; c < 3; ++c)
                if (fz[c]) f[c] = (T)0;
        }
        {
            const Quad<T> w0{clean ? (T)0 : m, clean ? (T)0 : p[0], clean ? (T)0 : p[1], clean ? (T)0 : p[2]};
            const Quad<T> w1{clean ? (T)0 : f[0], clean ? (T)0 : f[1], clean ? (T)0 : f[2], (T)0};
            *reinterpret_cast<Quad<T>*>(nd.acc + 8 * i) = w0;
            *reinterpret_cast<Quad<T>*>(nd.acc + 8 * i + 4) = w1;
        }
#pragma unroll
        for (int c = 0; c < 3; ++c)
            if (vset[c]) nd.vel[c * nn + i] = v[c];
        if (fx & 2u) nd.ftemp[nn + i] += ft_y;
        const bool has = m > mass_min;
        Quad<T> r, pm;
        r.x = has ? f[0] / m : (T)0;
        r.y = has ? f[1] / m : (T)0;
        r.z = has ? f[2] / m : (T)0;
        r.w = has ? (T)1 : (T)0;
        pm.x = p[0];
        pm.y = p[1];
        pm.z = p[2];
        pm.w = m;
        *reinterpret_cast<Quad<T>*>(nd.rec + 8 * i) = r;
        *reinterpret_cast<Quad<T>*>(nd.rec + 8 * i + 4) = pm;
        *reinterpret_cast<Quad<T>*>(nd.q + 4 * i) = Quad<T>{(T)0, (T)0, (T)0, (T)0};  // for pass 1's remap sums
    }
    work_add<T>(work, w_dc, w_fr, dtd);
}

// The node work between pass 1 and pass 2, in registers: the remap v += q/m
// (:559-560; phase A cleared q before pass 1 summed it), displacement
// control and BC (:573-599) in the path's order, then the record (p/m,
// m > m_min, v).  The claims are cleared after this last use (every claimed
// node is active: platen particles take part in P2G).  clean: a step whose
// node values nobody sees (not the last of an advance; pass 2 reads only the
// records) leaves the node zeroed as the next step's grid reset would
// (ResetGrid, …MPLocks.cpp:4-22), so that step needs no reset pass.
template <typename T>
__global__ void __launch_bounds__(256, 4) k_node_phase_b(NView<T> nd, int contact, const unsigned* __restrict__ dclist, int ndc,
                               const T* __restrict__ pvel, long long np, T mass_min, int clean, int vel_zero) {
    const long long nn = nd.nn;
    NODE_LOOP_AHEAD(nd, i) {
        const unsigned st = nd.state[i];
        if (!nd.alist && !(st & 1u)) continue;  // the list holds active nodes only
        const Quad<T> pm = ld_quad(nd.rec + 8 * i + 4);  // phase A's momentum and mass
        const T m = pm.w;
        const bool has = m > mass_min;
        const unsigned fx = nd.fixed[i];
        // vel_zero: the step began from a grid whose every nonzero node was in
        // the last active list (not an upload), so a node's velocity is zero
        // here unless phase A set it, which it does on fixed or claimed nodes only
        const bool vel_set = !vel_zero || fx != 0u || (st & NODE_CLAIMED);
        T v[3], p[3] = {pm.x, pm.y, pm.z};
        const Quad<T> q4 = ld_quad(nd.q + 4 * i);  // cleared by phase A, summed by pass 1
        const T q[3] = {q4.x, q4.y, q4.z};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            v[c] = vel_set ? nd.vel[c * nn + i] : (T)0;
            if (has) v[c] = v[c] + q[c] / m;
        }
        unsigned own[3] = {0u, 0u, 0u};
        if (ndc && (st & NODE_CLAIMED)) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (contact && a > 0) {  // one claim word for the three axes (k_dc_claim)
                    own[a] = own[0];
                    continue;
                }
                own[a] = nd.owner[a * nn + i];
                if (own[a]) nd.owner[a * nn + i] = 0u;  // the claims' last use this step: clean for the next
            }
        }
        bool vset[3] = {false, false, false}, fz[3] = {false, false, false};
        if (!contact) node_dc_regs<T>(own, dclist, pvel, np, m, v, vset, p, fz);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (fx & (1u << c)) {
                v[c] = (T)0;
                p[c] = (T)0;
                fz[c] = true;
            }
        }
        if (contact) node_dc_regs<T>(own, dclist, pvel, np, m, v, vset, p, fz);
        Quad<T> r, vq;
        r.x = has ? p[0] / m : (T)0;
        r.y = has ? p[1] / m : (T)0;
        r.z = has ? p[2] / m : (T)0;
        r.w = has ? (T)1 : (T)0;
        vq.x = v[0];
        vq.y = v[1];
        vq.z = v[2];
        vq.w = (T)0;
        *reinterpret_cast<Quad<T>*>(nd.rec + 8 * i) = r;
        *reinterpret_cast<Quad<T>*>(nd.rec + 8 * i + 4) = vq;
        if (clean) {  // phase A zeroed mass, momentum and force
#pragma unroll
            for (int c = 0; c < 3; ++c)
                if (vel_set) nd.vel[c * nn + i] = (T)0;
            if (fx & 2u) nd.ftemp[nn + i] = (T)0;  // the only reaction-force entry a step writes
            nd.state[i] = contact ? 0u : (st & ~(1u | NODE_CLAIMED));
        } else {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                nd.vel[c * nn + i] = v[c];
                nd.acc[8 * i + 1 + c] = p[c];
                if (fz[c]) nd.acc[8 * i + 4 + c] = (T)0;
            }
            if (st & NODE_CLAIMED) nd.state[i] = st & ~NODE_CLAIMED;
        }
    }
}

// TimeLine::getVelocity (TimeLine.h:33-46) is evaluated on the host each step
// and passed in as tv.
struct StepArgs {
    double dt;
    double mass_min;
    float dt_f;        // RN32(dt)
    float mass_min_f;  // mass_min rounded down to float (fps_float_threshold)
    double tv[3];
    const double* tv_dev;  // graph replay: the timeline velocity computed on the device (else tv)
    int has_timeline;
    int contact;
    // return-map network (FP32 form): materials it stands in for (bit per
    // material index), the fallback half-width (fraction of k0), the queue
    int sg_on;
    unsigned sg_mats;
    float sg_band;
    SurrogateQueue q;
    SurrogateAcc* sg_acc;
    // FP32 form: von Mises hardening particles whose trial yield function is
    // above -fb_below x k0 and that the network does not take (the states at
    // and past the yield surface, and elastic ones just below it, whose
    // elastic/plastic decision FP32 rounding could flip) run the exact map in
    // FP64 (cr_increment_wide).  Further below the surface the map is
    // D de, which FP32 gives to within an ulp of the FP64 value rounded.
    int fb_wide;
    float fb_below;
    // harvesting of return-map inputs (either form)
    int hv_on;
    unsigned hv_mats;
    float hv_band;
    float* hv_rows;
    unsigned* hv_count;
    long long hv_cap;
    // 1: also write the step's output-only particle field (the contact path's
    // strain rate, …_Contact.cpp:509, which no later step reads), as on the
    // last step of an advance
    int outputs;
};

// Where pass 2 reads a particle's fields from: its arrays in global memory
// (DirectSrc), or the block's copies in shared memory (StagedSrc below).
// Values written by the same step are always read back from global memory.
template <typename T>
struct DirectSrc {
    __device__ __forceinline__ unsigned pflags(const PView<T>& P, long long p) const { return P.pflags[p]; }
    __device__ __forceinline__ unsigned sid(const PView<T>& P, long long p) const { return P.sid[p]; }
    __device__ __forceinline__ unsigned key(const unsigned* keys, long long p) const { return keys[p]; }
    __device__ __forceinline__ int material(const PView<T>& P, long long p) const { return P.material[p]; }
    __device__ __forceinline__ T vol0(const PView<T>& P, long long p) const { return P.vol0[p]; }
    __device__ __forceinline__ T backstress(const PView<T>& P, long long p) const { return P.backstress[p]; }
    __device__ __forceinline__ float loc(const PView<T>& P, int k, long long p) const { return P.loc[k * P.n + p]; }
    __device__ __forceinline__ T F(const PView<T>& P, int k, long long p) const { return P.F[k * P.n + p]; }
    __device__ __forceinline__ T stress(const PView<T>& P, int k, long long p) const { return P.stress[k * P.n + p]; }
    __device__ __forceinline__ T strain(const PView<T>& P, int k, long long p) const { return P.strain[k * P.n + p]; }
    __device__ __forceinline__ T eps_p(const PView<T>& P, int k, long long p) const { return P.eps_p[k * P.n + p]; }
    __device__ __forceinline__ double pos(const PView<T>& P, int k, long long p) const { return P.pos[k * P.n + p]; }
    __device__ __forceinline__ double e_strain(const PView<T>& P, long long p) const { return P.e_strain[p]; }
    __device__ __forceinline__ double e_plastic(const PView<T>& P, long long p) const { return P.e_plastic[p]; }
};

__device__ __forceinline__ uint32_t shared_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Bounded wait for an mbarrier phase: false, with the error bit set, when it
// does not complete within 2^22 polls.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned* err) {
    for (int it = 0; it < (1 << 22); ++it) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    atomicOr(err, ERR_WAIT_TIMEOUT);
    return false;
}

// The FP32 pass 2's particle fields for one block of BS particles [p0, p0 + BS)
// in shared memory, brought in by bulk copies (cp.async.bulk) that all start
// at once and complete on one mbarrier, so the block's particle reads wait
// for one memory round trip instead of one per dependent load.  One segment
// per (field, component): BS elements plus 16 bytes, copied from the 16-byte
// boundary at or below the block's first element (component k of an n-element
// array starts (k n es) mod 16 bytes into its segment).  A block may stage
// only if p0 + BS + 16 <= n (every copy then stays inside its array) and
// every array starts on a 16-byte boundary.
template <int BS>
struct Pass2Stage {
    static constexpr int SEG1 = BS + 16, SEG2 = 2 * BS + 16, SEG4 = 4 * BS + 16, SEG8 = 8 * BS + 16;
    static constexpr int O_FLAGS = 0, O_SID = O_FLAGS + SEG1, O_KEYS = O_SID + SEG2, O_MAT = O_KEYS + SEG4;
    static constexpr int O_VOL0 = O_MAT + SEG4, O_BACK = O_VOL0 + SEG4, O_LOC = O_BACK + SEG4;
    static constexpr int O_F = O_LOC + 3 * SEG4, O_STRESS = O_F + 9 * SEG4, O_STRAIN = O_STRESS + 6 * SEG4;
    static constexpr int O_EPSP = O_STRAIN + 6 * SEG4, O_POS = O_EPSP + 6 * SEG4, O_ES = O_POS + 3 * SEG8;
    static constexpr int O_EP = O_ES + SEG8, BYTES = O_EP + SEG8;
    static constexpr int NSEG = 41;  // flags, sid, keys, material, vol0, back stress, 3 loc, 9 F, 3 x 6 tensors, 3 pos, 2 energies
    static constexpr int SMEM = BYTES + 16;  // and the mbarrier

    static __device__ __forceinline__ bool usable(const PView<float>& P, const unsigned* keys, long long p0) {
        const unsigned long long a = (unsigned long long)P.pflags | (unsigned long long)P.sid |
                                     (unsigned long long)keys | (unsigned long long)P.material |
                                     (unsigned long long)P.vol0 | (unsigned long long)P.backstress |
                                     (unsigned long long)P.loc | (unsigned long long)P.F |
                                     (unsigned long long)P.stress | (unsigned long long)P.strain |
                                     (unsigned long long)P.eps_p | (unsigned long long)P.pos |
                                     (unsigned long long)P.e_strain | (unsigned long long)P.e_plastic;
        const bool all = P.pflags && keys && P.material && P.vol0 && P.backstress && P.loc && P.F && P.stress &&
                         P.strain && P.eps_p && P.pos && P.e_strain && P.e_plastic;
        return all && (a & 15ull) == 0 && p0 + BS + 16 <= P.n;
    }
    // segment i: its array, element size, component and shared offset
    static __device__ __forceinline__ void segment(int i, const PView<float>& P, const unsigned* keys, const void*& base,
                                                   int& es, int& k, int& off) {
        k = 0;
        if (i == 0) { base = P.pflags; es = 1; off = O_FLAGS; }
        else if (i == 1) { base = P.sid; es = 2; off = O_SID; }
        else if (i == 2) { base = keys; es = 4; off = O_KEYS; }
        else if (i == 3) { base = P.material; es = 4; off = O_MAT; }
        else if (i == 4) { base = P.vol0; es = 4; off = O_VOL0; }
        else if (i == 5) { base = P.backstress; es = 4; off = O_BACK; }
        else if (i < 9) { base = P.loc; es = 4; k = i - 6; off = O_LOC; }
        else if (i < 18) { base = P.F; es = 4; k = i - 9; off = O_F; }
        else if (i < 24) { base = P.stress; es = 4; k = i - 18; off = O_STRESS; }
        else if (i < 30) { base = P.strain; es = 4; k = i - 24; off = O_STRAIN; }
        else if (i < 36) { base = P.eps_p; es = 4; k = i - 30; off = O_EPSP; }
        else if (i < 39) { base = P.pos; es = 8; k = i - 36; off = O_POS; }
        else if (i == 39) { base = P.e_strain; es = 8; off = O_ES; }
        else { base = P.e_plastic; es = 8; off = O_EP; }
        off += k * (BS * es + 16);
    }
    // bytes the block's copies deliver (no specimen ids with one specimen)
    static __device__ __forceinline__ unsigned tx_bytes(const PView<float>& P) {
        return (unsigned)(BYTES - (P.sid ? 0 : SEG2));
    }
    // issue segment i's copy (called by the lanes of one warp)
    static __device__ __forceinline__ void copy(int i, const PView<float>& P, const unsigned* keys, long long p0,
                                                unsigned char* sm, uint32_t bar) {
        const void* base;
        int es, k, off;
        segment(i, P, keys, base, es, k, off);
        if (!base) return;
        const unsigned long long src = ((unsigned long long)base + (unsigned long long)(k * P.n + p0) * es) & ~15ull;
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                shared_addr(sm + off)),
            "l"(src), "r"((unsigned)(BS * es + 16)), "r"(bar)
            : "memory");
    }
};

// Reads from a Pass2Stage: thread t's element of component k sits (k n es) mod
// 16 bytes plus t es into the component's segment.
template <int BS>
struct StagedSrc {
    using S = Pass2Stage<BS>;
    const unsigned char* sm;
    template <typename E, int OFF, int ES>
    __device__ __forceinline__ E at(const PView<float>& P, int k) const {
        const unsigned mis = ((unsigned)k * (unsigned)(P.n * ES)) & 15u;
        return *reinterpret_cast<const E*>(sm + OFF + k * (BS * ES + 16) + mis + threadIdx.x * ES);
    }
    __device__ __forceinline__ unsigned pflags(const PView<float>&, long long) const { return sm[S::O_FLAGS + threadIdx.x]; }
    __device__ __forceinline__ unsigned sid(const PView<float>& P, long long) const { return at<uint16_t, S::O_SID, 2>(P, 0); }
    __device__ __forceinline__ unsigned key(const unsigned*, long long) const {
        return *reinterpret_cast<const unsigned*>(sm + S::O_KEYS + 4 * threadIdx.x);
    }
    __device__ __forceinline__ int material(const PView<float>& P, long long) const { return at<int, S::O_MAT, 4>(P, 0); }
    __device__ __forceinline__ float vol0(const PView<float>& P, long long) const { return at<float, S::O_VOL0, 4>(P, 0); }
    __device__ __forceinline__ float backstress(const PView<float>& P, long long) const {
        return at<float, S::O_BACK, 4>(P, 0);
    }
    __device__ __forceinline__ float loc(const PView<float>& P, int k, long long) const { return at<float, S::O_LOC, 4>(P, k); }
    __device__ __forceinline__ float F(const PView<float>& P, int k, long long) const { return at<float, S::O_F, 4>(P, k); }
    __device__ __forceinline__ float stress(const PView<float>& P, int k, long long) const {
        return at<float, S::O_STRESS, 4>(P, k);
    }
    __device__ __forceinline__ float strain(const PView<float>& P, int k, long long) const {
        return at<float, S::O_STRAIN, 4>(P, k);
    }
    __device__ __forceinline__ float eps_p(const PView<float>& P, int k, long long) const {
        return at<float, S::O_EPSP, 4>(P, k);
    }
    __device__ __forceinline__ double pos(const PView<float>& P, int k, long long) const {
        return at<double, S::O_POS, 8>(P, k);
    }
    __device__ __forceinline__ double e_strain(const PView<float>& P, long long) const { return at<double, S::O_ES, 8>(P, 0); }
    __device__ __forceinline__ double e_plastic(const PView<float>& P, long long) const { return at<double, S::O_EP, 8>(P, 0); }
};

// Apply a constitutive increment o to particle p (stress, plastic strain,
// back stress, energies; …MPLocks.cpp:246-270, contact …_Contact.cpp:486-525).
// The step's energy increments are summed in the form's type and added once
// to the FP64 energy accumulators.
template <typename T, class SRC = DirectSrc<T>>
__device__ __forceinline__ void apply_increment(const PView<T>& P, long long p, const T sig[6], const T e[6],
                                                const CrOut<T>& o, T V, T R, int contact, double dt,
                                                const SRC& src = SRC{}) {
    const long long np = P.n;
    T dEs = 0, dEp = 0;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        T sn = sig[k] + o.dsig[k];
        P.stress[k * np + p] = sn;
        P.eps_p[k * np + p] = src.eps_p(P, k, p) + o.deps_p[k];
        if (!contact) {
            T mid = sn - (T)0.5 * o.dsig[k];
            dEs += mid * e[k] * V;
            dEp += mid * o.deps_p[k] * V;
        } else {
            dEs += sn * e[k] * V;
            dEp += sn * o.deps_p[k] * V;
        }
    }
    double es = src.e_strain(P, p) + fps_f2d_form(dEs);
    P.e_strain[p] = es;
    if (!contact) {
        P.e_strain_ti[p] += es * dt;
        if (es > P.e_strain_max[p]) P.e_strain_max[p] = es;
    }
    P.e_plastic[p] = src.e_plastic(P, p) + fps_f2d_form(dEp);
    P.backstress[p] = R + o.dR;
}

// Trial yield function of the von Mises hardening map (…_VonMisesHardening.cpp:20-46):
// sqrt(J2) of the elastic trial stress minus the radius k0 + R/sqrt 2.
template <typename T>
__device__ __forceinline__ T vmh_trial(const MatConst& m, T R, const T sig[6], const T e[6]) {
    T d[6];
    trial_increment<T>(m, e, d);
    T tr[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) tr[i] = sig[i] + d[i];
    const T a01 = tr[0] - tr[1], a12 = tr[1] - tr[2], a20 = tr[2] - tr[0];
    T J2 = (T)(1.0 / 6.0) * a01 * a01;
    J2 += (T)(1.0 / 6.0) * a12 * a12;
    J2 += (T)(1.0 / 6.0) * a20 * a20;
    J2 += tr[3] * tr[3];
    J2 += tr[4] * tr[4];
    J2 += tr[5] * tr[5];
    return sqrt(J2) - (form_const<T>(m.k0, m.fk0) + R * (T)0.70710678118654752440);
}

// warp-aggregated increment of a device counter; returns this lane's slot
__device__ __forceinline__ unsigned warp_slot(unsigned* counter) {
    const unsigned m = __activemask();
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(counter, (unsigned)__popc(m));
    base = __shfl_sync(m, base, leader);
    return base + __popc(m & ((1u << lane) - 1u));
}

// The particle arrays pass 2 reads, one per thread of a block's first warps:
// prefetched into L2 for the block's particle range while the warps gather
// the node records.
template <typename T>
__device__ __forceinline__ void pass2_prefetch(const PView<T>& P, long long p0, int cnt, int contact) {
    const int t = threadIdx.x;
    const long long n = P.n;
    const void* base = nullptr;
    int es = (int)sizeof(T);
    long long comp = 0;
    if (t < 3) {
        base = P.pos;
        es = 8;
        comp = t;
    } else if (t < 12) {
        base = P.F;
        comp = t - 3;
    } else if (t < 18) {
        base = P.stress;
        comp = t - 12;
    } else if (t < 24) {
        base = P.strain;
        comp = t - 18;
    } else if (t < 30) {
        base = P.eps_p;
        comp = t - 24;
    } else if (t == 30) {
        base = P.vol0;
    } else if (t == 31 && !contact) {  // the contact path writes V before reading it
        base = P.vol;
    } else if (t == 32) {
        base = P.backstress;
    } else if (t == 33) {
        base = P.e_strain;
        es = 8;
    } else if (t == 34) {
        base = P.e_plastic;
        es = 8;
    } else if (t == 35) {
        base = P.material;
        es = 4;
    } else if (t == 36) {
        base = P.pflags;
        es = 1;
    } else if (t == 37 && !contact) {
        base = P.e_strain_ti;
        es = 8;
    } else if (t == 38 && !contact) {
        base = P.e_strain_max;
        es = 8;
    }
    if (base) prefetch_l2((const char*)base + comp * n * es, es, n, p0, cnt);
}

// ---------------------------------------------------------------------------
// G2P pass 2 + constitutive update + platen (G2P_P2_SmallStrain,
// …MPLocks.cpp:175-280; contact …_Contact.cpp:438-525 and :531-540).
// One thread per particle in index order (coalesced particle streams).  At
// the end each particle also computes the cell key (and, in the FP32 form,
// the cell-local coordinate) of its new position for the next step, so the
// next step needs no separate key pass: `keys` is read (this step) and
// rewritten (next step), `keys_next` receives the next step's sort input.
// ---------------------------------------------------------------------------
// The large-strain pass 2's update of one particle after its gather
// (G2P_P2_LargeStrain, …MPLocks.cpp:311-435; FP64 form): the stress is reset,
// the logarithmic strains of F F^T (total, from the old F), of the trial
// elastic gradient dF F_e and of the increment dF are formed, the
// constitutive map takes zero stress and the trial elastic strain and returns
// the Kirchhoff stress, F_e becomes the exponential of the elastic strain,
// F = F dF, and stress = Kirchhoff / det F.  Energies add stress x increment x
// V component by component, as the reference does.
template <typename T>
__device__ __forceinline__ void large_strain_update(const PView<T>& P, long long p, const T Lt[9], double dt,
                                                    const MatConst* __restrict__ mats, int nmat, unsigned* err) {
    if constexpr (sizeof(T) == 8) {
        const long long np = P.n;
#pragma unroll
        for (int k = 0; k < 6; ++k) P.stress[k * np + p] = 0.0;
        double dF[9], F[9], Fe[9];
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int r = 0; r < 3; ++r) dF[3 * c + r] = (c == r ? 1.0 : 0.0) + (double)Lt[3 * c + r] * dt;
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            F[k] = P.F[k * np + p];
            Fe[k] = P.Fe[k * np + p];
        }
        double et[6], ee[6], einc[6], Fet[9];
        half_log_voigt(F, et);
        mat3_mul(dF, Fe, Fet);
        half_log_voigt(Fet, ee);
        half_log_voigt(dF, einc);
        const int mi = P.material[p];
        if (!(mi >= 0 && mi < nmat)) {
            atomicOr(err, ERR_BAD_MATERIAL);
            return;
        }
        const double zero[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        CrOut<double> o;
        cr_increment<double>(mats[mi], (double)P.backstress[p], zero, ee, o);
        double el[6], E[9], Fen[9], Fn[9];
#pragma unroll
        for (int k = 0; k < 6; ++k) el[k] = ee[k] - o.deps_p[k];
        E[0] = el[0];
        E[4] = el[1];
        E[8] = el[2];
        E[1] = E[3] = 0.5 * el[3];
        E[5] = E[7] = 0.5 * el[4];
        E[2] = E[6] = 0.5 * el[5];
        mat3_exp8(E, Fen);
        mat3_mul(F, dF, Fn);
        const double det = Kinematics<double>::det(Fn);
        const double V = det * (double)P.vol0[p];
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            P.Fe[k * np + p] = Fen[k];
            P.F[k * np + p] = Fn[k];
        }
        P.vol[p] = V;
        double es = P.e_strain[p], ep = P.e_plastic[p];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const double sn = (1.0 / det) * o.dsig[k];
            P.strain[k * np + p] = et[k];
            P.stress[k * np + p] = sn;
            P.eps_p[k * np + p] += o.deps_p[k];
            es += sn * einc[k] * V;
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) ep += (1.0 / det) * o.dsig[k] * o.deps_p[k] * V;
        P.e_strain[p] = es;
        P.e_plastic[p] = ep;
        P.backstress[p] += o.dR;
    }
}

// One particle of pass 2; returns the new cell key (u: the new cell-local
// coordinate; queued: its stress increment waits for the network).
template <typename T, int BATCH, bool LS = false, class SRC = DirectSrc<T>>
__device__ __forceinline__ unsigned pass2_particle(const PView<T>& P, const NView<T>& nd, const Geom& g,
                                                   unsigned* __restrict__ keys, unsigned* __restrict__ keys_next,
                                                   const MatConst* __restrict__ mats, int nmat, const StepArgs& a,
                                                   unsigned* err, long long p, float u[3], bool& queued,
                                                   const SRC& src = SRC{}) {
    const long long np = P.n, nn = nd.nn;
    queued = false;
    const unsigned fl = src.pflags(P, p);
    const T dt = form_const<T>(a.dt, a.dt_f);
    const T mass_min = form_const<T>(a.mass_min, a.mass_min_f);
    const bool skip = a.contact && (fl & 8u);
    const Geom& gs = (g.nspec > 1) ? g.tab[src.sid(P, p)] : g;
    if (!skip) {
        unsigned key = src.key(keys, p);
        double x[3] = {src.pos(P, 0, p), src.pos(P, 1, p), src.pos(P, 2, p)};
        T L[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) L[k] = 0;
        if (key < g.key_max) {
            int b[3];
            key_to_base(key, gs, b);
            Bases<T> B;
            if constexpr (sizeof(T) == 4) {
                const float ul[3] = {src.loc(P, 0, p), src.loc(P, 1, p), src.loc(P, 2, p)};
                B.init_local(gs, ul);
            } else {
                particle_bases<T>(P, gs, p, b, B);
            }
            const double ddt = a.dt;
            // FP32 form: the displacement sum N (p/m) is formed in FP32 and
            // added to the FP64 position once; FP64 form: added per corner
            // as the reference does (…MPLocks.cpp:197-198).
            T disp[3] = {0, 0, 0};
            // BATCH: four corners' records are requested before any is used
            // (two round trips to memory instead of eight, at more registers);
            // sums run in corner order either way.  The FP32 form unrolls the
            // corners (fewer instructions per corner)
            const CellNodes cn = cell_nodes(gs, b);
#pragma unroll(BATCH ? 2 : (sizeof(T) == 4 ? 8 : 1))
            for (int h = 0; h < (BATCH ? 2 : 8); ++h) {
                constexpr int W = BATCH ? 4 : 1;
                Quad<T> rq[W], vq[W];
                bool in[W];
#pragma unroll
                for (int j = 0; j < W; ++j) {
                    const long long nid = cell_node(cn, W * h + j);
                    in[j] = (cn.mask >> (W * h + j)) & 1u;
                    const Quad<T> z{(T)0, (T)0, (T)0, (T)0};
                    rq[j] = z;
                    vq[j] = z;
                    if (in[j]) ld_record(nd.rec + 8 * nid, rq[j], vq[j]);
                }
#pragma unroll
                for (int j = 0; j < W; ++j) {
                    if (!in[j]) continue;
                    T N, G[3];
                    B.corner(W * h + j, N, G);
                    if (rq[j].w != (T)0) {  // m > mass_min
                        const T rr[3] = {rq[j].x, rq[j].y, rq[j].z};
                        if constexpr (sizeof(T) == 4) {
#pragma unroll
                            for (int c = 0; c < 3; ++c) disp[c] += N * rr[c];
                        } else {
#pragma unroll
                            for (int c = 0; c < 3; ++c) x[c] = x[c] + (double)(N * rr[c]) * ddt;
                        }
                    }
                    const T vi[3] = {vq[j].x, vq[j].y, vq[j].z};
                    // outerProduct(v_i, grad N): column c, row r = v_i[r] * G[c]
#pragma unroll
                    for (int c = 0; c < 3; ++c)
#pragma unroll
                        for (int r = 0; r < 3; ++r) L[3 * c + r] += vi[r] * G[c];
                }
            }
            if constexpr (sizeof(T) == 4) {
#pragma unroll
                for (int c = 0; c < 3; ++c) x[c] += fps_f2d(disp[c] * dt);
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) P.pos[c * np + p] = x[c];
        }
        if constexpr (LS) {
            large_strain_update(P, p, L, (double)dt, mats, nmat, err);
        } else {
        // strain increment: diagonal from dF = I + L dt (form-specific, see
        // Kinematics), off-diagonal (L_ij + L_ji) dt in Voigt engineering shear
        T Ldt[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) Ldt[k] = L[k] * dt;
        T e[6];
        e[0] = Kinematics<T>::strain_diag(Ldt[0]);
        e[1] = Kinematics<T>::strain_diag(Ldt[4]);
        e[2] = Kinematics<T>::strain_diag(Ldt[8]);
        e[3] = Ldt[1] + Ldt[3];
        e[4] = Ldt[5] + Ldt[7];
        e[5] = Ldt[6] + Ldt[2];
        int mi = src.material(P, p);
        T F[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) F[k] = src.F(P, k, p);
        T Fn[9];
        Kinematics<T>::update(a.contact != 0, F, L, Ldt, dt, Fn);
        if (a.contact) {
            // contact: strain, F and V are updated before the material check (…_Contact.cpp:464-484)
#pragma unroll
            for (int k = 0; k < 6; ++k) P.strain[k * np + p] = src.strain(P, k, p) + e[k];
#pragma unroll
            for (int k = 0; k < 9; ++k) P.F[k * np + p] = Fn[k];
            P.vol[p] = Kinematics<T>::det(Fn) * src.vol0(P, p);
        }
        if (mi >= 0 && mi < nmat) {
            const MatConst& M = mats[mi];
            T sig[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) sig[k] = src.stress(P, k, p);
            T R = src.backstress(P, p);
            CrOut<T> o;
            // the network takes clearly plastic trial states of the materials it
            // was trained for; the band near the surface and elastic states stay
            // exact, the band (and every plastic state the network does not take)
            // in FP64
            queued = false;
            CrTrial<T> tr;
            cr_trial<T>(M, R, sig, e, tr);
            bool wide = false;
            if constexpr (sizeof(T) == 4) {
                if (M.type == 4) {
                    const float f = sqrtf(tr.J2) - tr.rad;  // the trial yield function (…_VonMisesHardening.cpp:35-46)
                    if (a.sg_on && mi < 32 && ((a.sg_mats >> mi) & 1u)) {
                        queued = f >= a.sg_band * M.fk0;
                        if (!queued && f > 0.0f) {
                            const unsigned m = __activemask();
                            if ((threadIdx.x & 31) == __ffs(m) - 1) atomicAdd(&a.sg_acc->band, (unsigned long long)__popc(m));
                        }
                    }
                    wide = a.fb_wide && !queued && f > -a.fb_below * M.fk0;
                }
            }
            if (a.hv_on && mi < 32 && ((a.hv_mats >> mi) & 1u) && M.type == 4 &&
                vmh_trial<T>(M, R, sig, e) >= (T)a.hv_band * form_const<T>(M.k0, M.fk0)) {
                const unsigned slot = warp_slot(a.hv_count);
                if (slot < (unsigned long long)a.hv_cap) {
                    float* hr = a.hv_rows + (long long)slot * 13;
#pragma unroll
                    for (int k = 0; k < 6; ++k) {
                        hr[k] = (float)sig[k];
                        hr[7 + k] = (float)e[k];
                    }
                    hr[6] = (float)R;
                }
            }
            if (!queued) {
                if constexpr (sizeof(T) == 4) {
                    if (wide) {
                        CrOut<double> w;
                        cr_increment_wide(M, R, sig, e, w);
                        cr_narrow(w, o);
                    } else {
                        cr_return<T>(M, R, sig, e, tr, o);
                    }
                } else {
                    cr_return<T>(M, R, sig, e, tr, o);
                }
            }
            T V;
            if (!a.contact) {
#pragma unroll
                for (int k = 0; k < 9; ++k) P.F[k * np + p] = Fn[k];
                V = Kinematics<T>::det(Fn) * src.vol0(P, p);
                P.vol[p] = V;
#pragma unroll
                for (int k = 0; k < 6; ++k) P.strain[k * np + p] = src.strain(P, k, p) + e[k];
            } else {
                V = P.vol[p];
                if (a.outputs) {
#pragma unroll
                    for (int k = 0; k < 6; ++k) P.strain_rate[k * np + p] = e[k] / dt;
                }
            }
            if (queued) {
                if constexpr (sizeof(T) == 4) {
                    const unsigned slot = warp_slot(a.q.count);
                    if (slot < (unsigned long long)a.q.cap) {
                        float* qi = a.q.in + (long long)slot * 13;
#pragma unroll
                        for (int k = 0; k < 6; ++k) {
                            qi[k] = sig[k];
                            qi[7 + k] = e[k];
                        }
                        qi[6] = R;
                        a.q.vol[slot] = V;
                        a.q.pidx[slot] = (unsigned)p;
                    }
                }
            } else {
                apply_increment<T>(P, p, sig, e, o, V, R, a.contact, a.dt, src);
            }
        } else if (!a.contact) {
            atomicOr(err, ERR_BAD_MATERIAL);
        }
        }
    }
    // platen timeline (…MPLocks.cpp:766-789; contact :531-540)
    if (fl & PF_IN_DC) {
        const double* tv = a.tv_dev ? a.tv_dev : a.tv;
        if (!a.contact) {
            if (a.has_timeline) {
#pragma unroll
                for (int c = 0; c < 3; ++c)
                    if (fl & (1u << c)) P.vel[c * np + p] = (T)((double)P.dc_mult[p] * tv[c]);
            }
        } else {
            double vv[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                vv[c] = a.has_timeline ? (double)P.dc_mult[p] * tv[c] : (double)P.vel[c * np + p];
                P.vel[c * np + p] = (T)vv[c];
                P.pos[c * np + p] += vv[c] * a.dt;
            }
        }
    }
    // the next step's cell key (and FP32 cell-local coordinate) from the new position
    const double xn[3] = {P.pos[p], P.pos[np + p], P.pos[2 * np + p]};
    const unsigned nk = particle_key(gs, xn, u, err);
    keys[p] = nk;
    if (keys_next) keys_next[p] = nk;
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int c = 0; c < 3; ++c) P.loc[c * np + p] = u[c];
    }
    return nk;
}

// BS: the block size; the FP32 form asks for 1280 / BS blocks per SM (48
// registers: a few spill, and the extra resident warps hide more of the
// gathers' latency).
template <typename T, int BATCH, int BS>
__global__ void __launch_bounds__(BS, sizeof(T) == 4 ? 1280 / BS : 1) k_pass2(PView<T> P, NView<T> nd, Geom g, unsigned* __restrict__ keys,
                                               unsigned* __restrict__ keys_next, const MatConst* __restrict__ mats,
                                               int nmat, StepArgs a, unsigned* err) {
    const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (threadIdx.x < 64) pass2_prefetch<T>(P, blockIdx.x * (long long)blockDim.x, blockDim.x, a.contact);
    if (p >= P.n) return;
    float u[3];
    bool queued;
    pass2_particle<T, BATCH>(P, nd, g, keys, keys_next, mats, nmat, a, err, p, u, queued);
}

// FP32 pass 2 with the block's particle fields staged in shared memory
// (Pass2Stage): warp 0 issues the bulk copies, every thread waits once on the
// mbarrier, then runs pass2_particle reading from shared memory.  Blocks that
// cannot stage (the last ones, or unaligned arrays) read global memory.
// Blocks per SM: as many as the staging buffers fit (228 KB of shared memory,
// 1 KB reserved per block), which sets the register budget.
template <int BS>
constexpr int pass2_staged_blocks() {
    return (228 * 1024) / (Pass2Stage<BS>::SMEM + 1024);
}

template <int BS>
__global__ void __launch_bounds__(BS, pass2_staged_blocks<BS>()) k_pass2_staged(PView<float> P, NView<float> nd, Geom g,
                                                               unsigned* __restrict__ keys,
                                                               unsigned* __restrict__ keys_next,
                                                               const MatConst* __restrict__ mats, int nmat,
                                                               StepArgs a, unsigned* err) {
    using S = Pass2Stage<BS>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int t = threadIdx.x;
    const long long p0 = blockIdx.x * (long long)BS, p = p0 + t;
    float u[3];
    bool queued;
    if (!S::usable(P, keys, p0)) {
        if (t < 64) pass2_prefetch<float>(P, p0, BS, a.contact);
        if (p < P.n) pass2_particle<float, 0>(P, nd, g, keys, keys_next, mats, nmat, a, err, p, u, queued);
        return;
    }
    const uint32_t bar = shared_addr(smem_raw + S::BYTES);
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (t < 32) {
        if (t == 0)
            asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n" ::"r"(bar),
                         "r"(S::tx_bytes(P))
                         : "memory");
        __syncwarp();
        for (int i = t; i < S::NSEG; i += 32) S::copy(i, P, keys, p0, smem_raw, bar);
    }
    if (!mbar_wait(bar, 0, err)) {
        mbar_wait(bar, 0, err);  // once more (bounded) for copies still in flight, then leave
        return;
    }
    pass2_particle<float, 0, false, StagedSrc<BS>>(P, nd, g, keys, keys_next, mats, nmat, a, err, p, u, queued,
                                                   StagedSrc<BS>{smem_raw});
}

// The large-strain pass 2 (non-contact loop, FP64 form; the reference ships
// it disabled, …MPLocks.cpp:605, and MPM_OPT_LARGE_STRAIN switches it on).
template <int BS>
__global__ void __launch_bounds__(BS) k_pass2_ls(PView<double> P, NView<double> nd, Geom g, unsigned* __restrict__ keys,
                                                 unsigned* __restrict__ keys_next, const MatConst* __restrict__ mats,
                                                 int nmat, StepArgs a, unsigned* err) {
    const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    float u[3];
    bool queued;
    pass2_particle<double, 0, true>(P, nd, g, keys, keys_next, mats, nmat, a, err, p, u, queued);
}

// ---------------------------------------------------------------------------
// Contact detection (…_Contact.cpp:152-237), bit-exact.
// Node mass gradients sum grad N m_p over all particles; the reference adds
// them in particle index order (one thread), and the max-norm selection that
// follows is sensitive to the last bit.  Only nodes adjacent to surface
// particles are ever read, so those nodes are summed here by one thread each,
// merging the (index-ordered) particle ranges of the eight surrounding cells
// in index order, with the reference's exact per-pair gradient.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_contact_need(PView<T> P, const unsigned* __restrict__ keys, Geom g, unsigned* __restrict__ need,
                               const unsigned* __restrict__ surf, int nsurf) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nsurf) return;
    const long long p = surf[t];
    unsigned key = keys[p];
    if (key >= g.key_max) return;
    const Geom& gs = spec_geom(g, P.sid, p);
    int b[3];
    key_to_base(key, gs, b);
    for (int k = 0; k < 8; ++k) {
        long long nid = corner_node(gs, b, k);
        if (nid >= 0) need[nid] = 1u;
    }
}

// Compact the needed nodes into a list (order irrelevant: nodes are independent).
static __global__ void k_contact_compact(const unsigned* __restrict__ need, long long nn, unsigned* __restrict__ list,
                                         unsigned* __restrict__ count) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    bool take = i < nn && need[i];
    unsigned m = __ballot_sync(FULL_MASK, take);
    if (!m) return;
    int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(count, (unsigned)__popc(m));
    base = __shfl_sync(m, base, leader);
    if (take) list[base + __popc(m & ((1u << lane) - 1u))] = (unsigned)i;
}

// One warp per needed node: gather the particle ids of the eight surrounding
// cells into shared memory, rank them by id, compute each pair's exact
// grad N * m in parallel, then add them in id order on one lane.  Nodes with
// more than CG_CAP contributors take the one-lane merge below.
constexpr int CG_WARPS = 4;
constexpr int CG_CAP = 256;

template <typename T>
__device__ __noinline__ void mass_gradient_merge(const PView<T>& P, const Geom& g, const int node[3],
                                                 const unsigned* __restrict__ perm, const unsigned cs[8],
                                                 const unsigned ce[8], double gsum[3]) {
    const long long np = P.n;
    unsigned cur[8], end[8];
    for (int k = 0; k < 8; ++k) {
        cur[k] = cs[k];
        end[k] = ce[k];
    }
    gsum[0] = gsum[1] = gsum[2] = 0.0;
    while (true) {
        int best = -1;
        unsigned bp = 0xffffffffu;
        for (int c = 0; c < 8; ++c) {
            if (cur[c] < end[c]) {
                unsigned pp = perm[cur[c]];
                if (pp < bp) {
                    bp = pp;
                    best = c;
                }
            }
        }
        if (best < 0) break;
        cur[best]++;
        double x[3] = {P.pos[bp], P.pos[np + bp], P.pos[2 * np + bp]};
        double G[3];
        exact_gradient(g, x, node, G);
        double m = (double)P.mass[bp];
        for (int c = 0; c < 3; ++c) gsum[c] = __dadd_rn(gsum[c], __dmul_rn(G[c], m));
    }
}

template <typename T>
__global__ void __launch_bounds__(CG_WARPS * 32) k_contact_mass_gradient(PView<T> P, NView<T> nd, Geom g,
                                                                         const unsigned* __restrict__ list,
                                                                         const unsigned* __restrict__ count,
                                                                         const unsigned* __restrict__ perm,
                                                                         const unsigned* __restrict__ cstart,
                                                                         const unsigned* __restrict__ cend) {
    __shared__ unsigned s_id[CG_WARPS][CG_CAP];
    __shared__ double s_c[CG_WARPS][CG_CAP][3];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long np = P.n, nn = nd.nn;
    const unsigned total_nodes = *count;
    for (unsigned item = blockIdx.x * CG_WARPS + w; item < total_nodes; item += gridDim.x * CG_WARPS) {
        const long long i = list[item];
        const Geom& gs = node_geom(g, i);
        const long long il = i - gs.node_off;
        int node[3];
        node[0] = (int)(il % gs.nn[0]);
        node[1] = (int)((il / gs.nn[0]) % gs.nn[1]);
        node[2] = (int)(il / ((long long)gs.nn[0] * gs.nn[1]));
        // lanes 0..7: the eight surrounding cells (cell = node - {0,1}^3)
        unsigned s0 = 0, len = 0;
        if (lane < 8) {
            int cb[3] = {node[0] - ((lane >> 2) & 1), node[1] - ((lane >> 1) & 1), node[2] - (lane & 1)};
            unsigned key = gs.key_off + (unsigned)((cb[0] + 1) + gs.kd[0] * ((cb[1] + 1) + gs.kd[1] * (cb[2] + 1)));
            s0 = cstart[key];
            unsigned s1 = cend[key];
            len = s1 > s0 ? s1 - s0 : 0u;
        }
        // exclusive offsets of the segments
        unsigned off = len;
#pragma unroll
        for (int d = 1; d < 8; d <<= 1) {
            unsigned o = __shfl_up_sync(FULL_MASK, off, d);
            if (lane >= d) off += o;
        }
        const unsigned total = __shfl_sync(FULL_MASK, off, 7);
        off -= len;
        unsigned segs[8], offs[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            segs[k] = __shfl_sync(FULL_MASK, s0, k);
            offs[k] = __shfl_sync(FULL_MASK, off, k);
        }
        double gsum[3] = {0.0, 0.0, 0.0};
        if (total > (unsigned)CG_CAP) {
            if (lane == 0) {
                unsigned cs[8], ce[8];
                for (int k = 0; k < 8; ++k) {
                    cs[k] = segs[k];
                    ce[k] = segs[k] + ((k < 7 ? offs[k + 1] : total) - offs[k]);
                }
                mass_gradient_merge<T>(P, gs, node, perm, cs, ce, gsum);
            }
        } else {
            for (unsigned e = lane; e < total; e += 32) {
                int k = 0;
#pragma unroll
                for (int kk = 1; kk < 8; ++kk)
                    if (e >= offs[kk]) k = kk;
                s_id[w][e] = perm[segs[k] + (e - offs[k])];
            }
            __syncwarp();
            for (unsigned e = lane; e < total; e += 32) {
                const unsigned id = s_id[w][e];
                unsigned rank = 0;
                for (unsigned j = 0; j < total; ++j) rank += s_id[w][j] < id ? 1u : 0u;
                double x[3] = {P.pos[id], P.pos[np + id], P.pos[2 * np + id]};
                double G[3];
                exact_gradient(gs, x, node, G);
                const double m = (double)P.mass[id];
                s_c[w][rank][0] = __dmul_rn(G[0], m);
                s_c[w][rank][1] = __dmul_rn(G[1], m);
                s_c[w][rank][2] = __dmul_rn(G[2], m);
            }
            __syncwarp();
            if (lane < 3) {
                double acc = 0.0;
                for (unsigned e = 0; e < total; ++e) acc = __dadd_rn(acc, s_c[w][e][lane]);
                gsum[lane] = acc;
            }
        }
        if (total > (unsigned)CG_CAP) {
            if (lane == 0) {
#pragma unroll
                for (int c = 0; c < 3; ++c) nd.mg[c * nn + i] = gsum[c];
            }
        } else if (lane < 3) {
            nd.mg[lane * nn + i] = gsum[lane];
        }
        __syncwarp();
    }
}

// The contact kernels below run one thread per surface particle (a list
// compacted at upload).  FP64 form: the reference's uncontracted FP64
// arithmetic, bit-exact.  FP32 form: the same tests in FP32 (the flags only
// feed output, as in the reference, where nothing reads them back).
__device__ __forceinline__ float dot3f(const float a[3], const float b[3]) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// Surface particle normal: the corner gradient of largest norm, first wins on ties (:156-172).
template <typename T>
__global__ void k_contact_mp_gradient(PView<T> P, NView<T> nd, Geom g, const unsigned* __restrict__ keys,
                                      const unsigned* __restrict__ surf, int nsurf) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nsurf) return;
    const long long p = surf[t];
    const Geom& gs = spec_geom(g, P.sid, p);
    const long long np = P.n, nn = nd.nn;
    T gp[3] = {0, 0, 0};
    unsigned key = keys[p];
    if (key < g.key_max) {
        int b[3];
        key_to_base(key, gs, b);
        float best2 = 0.0f;
        for (int k = 0; k < 8; ++k) {
            long long nid = corner_node(gs, b, k);
            if (nid < 0) continue;
            T gi[3] = {nd.mg[nid], nd.mg[nn + nid], nd.mg[2 * nn + nid]};
            bool take;
            if constexpr (sizeof(T) == 8) {
                take = len3_rn(gi) > len3_rn(gp);
            } else {
                float l2 = dot3f(gi, gi);
                take = l2 > best2;
                if (take) best2 = l2;
            }
            if (take) {
                gp[0] = gi[0];
                gp[1] = gi[1];
                gp[2] = gi[2];
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) P.mp_mg[c * np + p] = gp[c];
}

// Reset the node mass gradient of active nodes (:177-186) and the normal claims.
template <typename T>
__device__ __forceinline__ void contact_reset_node(const NView<T>& nd, long long i) {
    nd.nowner[i] = 0u;
    if (!(nd.state[i] & 1u)) return;
    const long long nn = nd.nn;
#pragma unroll
    for (int c = 0; c < 3; ++c) nd.mg[c * nn + i] = 0.0;
}

template <typename T>
__global__ void k_contact_reset(NView<T> nd) {
    NODE_LOOP(nd, i) contact_reset_node<T>(nd, i);
}

// Node normal from surface particles with (x_i - x_p) . g_p > 0 (:191-210);
// the reference overwrites in index order, so the largest index wins.
template <typename T>
__global__ void k_contact_normal(PView<T> P, NView<T> nd, Geom g, const unsigned* __restrict__ keys,
                                 const unsigned* __restrict__ surf, int nsurf, int apply) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nsurf) return;
    const long long p = surf[t];
    const Geom& gs = spec_geom(g, P.sid, p);
    const long long np = P.n, nn = nd.nn;
    unsigned key = keys[p];
    if (key >= g.key_max) return;
    int b[3];
    key_to_base(key, gs, b);
    const T gp[3] = {P.mp_mg[p], P.mp_mg[np + p], P.mp_mg[2 * np + p]};
    for (int k = 0; k < 8; ++k) {
        long long nid = corner_node(gs, b, k);
        if (nid < 0) continue;
        int o3[3] = {(k >> 2) & 1, (k >> 1) & 1, k & 1};
        bool facing;
        if constexpr (sizeof(T) == 8) {
            double d[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) d[c] = __dadd_rn(node_coord(gs, c, b[c] + o3[c]), -P.pos[c * np + p]);
            facing = dot3_rn(d, gp) > 0.0;
        } else {
            // node minus particle from the cell-local coordinate: (o - u) h per axis
            float d[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) d[c] = ((float)o3[c] - P.loc[c * np + p]) * gs.hf[c];
            facing = dot3f(d, gp) > 0.0f;
        }
        if (!facing) continue;
        const unsigned who = (P.orig ? P.orig[p] : (unsigned)p) + 1u;  // the caller's particle order
        if (!apply) {
            atomicMax(&nd.nowner[nid], who);
        } else if (nd.nowner[nid] == who) {
#pragma unroll
            for (int c = 0; c < 3; ++c) nd.mg[c * nn + nid] = gp[c];
        }
    }
}

// Contact flags (:215-237): g_i . g_p >= 0.001 |g_i| |g_p| -> positive, <= -tol -> negative.
template <typename T>
__global__ void k_contact_flags(PView<T> P, NView<T> nd, Geom g, const unsigned* __restrict__ keys,
                                const unsigned* __restrict__ surf, int nsurf) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nsurf) return;
    const long long p = surf[t];
    const Geom& gs = spec_geom(g, P.sid, p);
    const long long np = P.n, nn = nd.nn;
    unsigned key = keys[p];
    if (key >= g.key_max) return;
    int b[3];
    key_to_base(key, gs, b);
    const T gp[3] = {P.mp_mg[p], P.mp_mg[np + p], P.mp_mg[2 * np + p]};
    double lp = 0.0;
    float lpf = 0.0f;
    if constexpr (sizeof(T) == 8)
        lp = len3_rn(gp);
    else
        lpf = sqrtf(dot3f(gp, gp));
    for (int k = 0; k < 8; ++k) {
        long long nid = corner_node(gs, b, k);
        if (nid < 0) continue;
        const T gi[3] = {nd.mg[nid], nd.mg[nn + nid], nd.mg[2 * nn + nid]};
        bool pos, neg;
        if constexpr (sizeof(T) == 8) {
            double tol = __dmul_rn(__dmul_rn(0.001, len3_rn(gi)), lp);
            double dd = dot3_rn(gi, gp);
            pos = dd >= tol;
            neg = !pos && dd <= -tol;
        } else {
            float tol = 0.001f * sqrtf(dot3f(gi, gi)) * lpf;
            float dd = dot3f(gi, gp);
            pos = dd >= tol;
            neg = !pos && dd <= -tol;
        }
        if (pos)
            atomicOr(&nd.state[nid], 4u);
        else if (neg)
            atomicOr(&nd.state[nid], 8u);
    }
}

// ---------------------------------------------------------------------------
// Console monitors (PhysicsEngine::reportConsole, PhysicsEngine.cpp:40-183).
// acc layout (doubles): 0-2 position sum, 3-5 momentum, 6 max |principal
// strain|, 7 max |principal stress|, 8-10 stress sum, 11-13 strain sum,
// 14 kinetic, 15 strain energy, 16 plastic energy, 17-19 reaction-force sum;
// counts (u64) follow at 24-28.
// ---------------------------------------------------------------------------
constexpr int MON_SLOTS = 32;

// ConstitutiveRelation::getPrincipal (ConstitutiveRelation_calculateState.cpp:160-196),
// largest |principal value|; NaN (hydrostatic or zero states) or Q > 0 give 0,
// as the reference's max update skips them.
__device__ __forceinline__ double principal_abs_max(const double s[6]) {
    const double I1 = s[0] + s[1] + s[2];
    double I2 = 0.0;
    I2 += s[0] * s[1];
    I2 += s[1] * s[2];
    I2 += s[0] * s[2];
    I2 -= s[3] * s[3];
    I2 -= s[4] * s[4];
    I2 -= s[5] * s[5];
    // symmetric matrix [[s0 s3 s5] [s3 s1 s4] [s5 s4 s2]], glm cofactor determinant
    const double m[9] = {s[0], s[3], s[5], s[3], s[1], s[4], s[5], s[4], s[2]};
    const double I3 = Kinematics<double>::det(m);
    const double Q = (3.0 * I2 - I1 * I1) / 9.0;
    const double R = (2.0 * I1 * I1 * I1 - 9.0 * I1 * I2 + 27.0 * I3) / 54.0;
    if (Q > 0.0) return 0.0;
    double T = R / sqrt(-Q * Q * Q);
    if (!(T == T)) return 0.0;
    T = fmin(fmax(T, -1.0), 1.0);
    const double th = acos(T), pi = 3.14159265359;  // _PI, Definitions.h:12
    double best = 0.0;
    for (int k = 0; k < 3; ++k) {
        double v = fabs(2.0 * sqrt(-Q) * cos((th + 2.0 * k * pi) / 3.0) + 1.0 / 3.0 * I1);
        if (v == v && v > best) best = v;
    }
    return best;
}

__device__ __forceinline__ void atomic_max_nonneg(double* a, double v) {
    atomicMax((unsigned long long*)a, (unsigned long long)__double_as_longlong(v));
}

template <typename T>
__global__ void __launch_bounds__(256) k_monitors(PView<T> P, const uint8_t* __restrict__ mask, double* acc) {
    __shared__ double sh[8][17];
    __shared__ unsigned long long shc[8][5];
    long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long np = P.n;
    double v[17];
#pragma unroll
    for (int k = 0; k < 17; ++k) v[k] = 0.0;
    unsigned long long cnt[5] = {0, 0, 0, 0, 0};
    if (p < np) {
        const unsigned mk = mask[p];
        const double m = (double)P.mass[p];
        double vel[3] = {(double)P.vel[p], (double)P.vel[np + p], (double)P.vel[2 * np + p]};
        if (mk & 1u) {
            for (int c = 0; c < 3; ++c) v[c] = P.pos[c * np + p];
            cnt[0] = 1;
        }
        if (mk & 2u) {
            for (int c = 0; c < 3; ++c) v[3 + c] = vel[c] * m;
            cnt[1] = 1;
        }
        double sg[6], ep[6];
        for (int c = 0; c < 6; ++c) {
            sg[c] = (double)P.stress[c * np + p];
            ep[c] = (double)P.strain[c * np + p];
        }
        if (mk & 4u) {
            v[6] = principal_abs_max(ep);
            v[7] = principal_abs_max(sg);
            cnt[2] = 1;
        }
        if (mk & 8u) {
            for (int c = 0; c < 3; ++c) {
                v[8 + c] = sg[c];
                v[11 + c] = ep[c];
            }
            cnt[3] = 1;
        }
        if (mk & 16u) {
            double sp = sqrt(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
            v[14] = 0.5 * m * (sp * sp);
            v[15] = P.e_strain[p];
            v[16] = P.e_plastic[p];
            cnt[4] = 1;
        }
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 17; ++k) {
        for (int off = 16; off > 0; off >>= 1) {
            double o = __shfl_down_sync(FULL_MASK, v[k], off);
            v[k] = (k == 6 || k == 7) ? fmax(v[k], o) : v[k] + o;
        }
    }
#pragma unroll
    for (int k = 0; k < 5; ++k)
        for (int off = 16; off > 0; off >>= 1) cnt[k] += __shfl_down_sync(FULL_MASK, cnt[k], off);
    if (lane == 0) {
        for (int k = 0; k < 17; ++k) sh[w][k] = v[k];
        for (int k = 0; k < 5; ++k) shc[w][k] = cnt[k];
    }
    __syncthreads();
    if (threadIdx.x < 17) {
        const int k = threadIdx.x;
        double s = sh[0][k];
        for (int ww = 1; ww < (int)(blockDim.x >> 5); ++ww) s = (k == 6 || k == 7) ? fmax(s, sh[ww][k]) : s + sh[ww][k];
        if (k == 6 || k == 7)
            atomic_max_nonneg(&acc[k], s);
        else
            atomicAdd(&acc[k], s);
    } else if (threadIdx.x >= 32 && threadIdx.x < 37) {
        const int k = threadIdx.x - 32;
        unsigned long long s = 0;
        for (int ww = 0; ww < (int)(blockDim.x >> 5); ++ww) s += shc[ww][k];
        atomicAdd((unsigned long long*)&acc[24 + k], s);
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_monitor_force(NView<T> nd, double* acc) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long nn = nd.nn;
    double f[3] = {0.0, 0.0, 0.0};
    if (i < nn)
        for (int c = 0; c < 3; ++c) f[c] = (double)nd.ftemp[c * nn + i];
    for (int c = 0; c < 3; ++c) {
        for (int off = 16; off > 0; off >>= 1) f[c] += __shfl_down_sync(FULL_MASK, f[c], off);
        if ((threadIdx.x & 31) == 0) atomicAdd(&acc[17 + c], f[c]);
    }
}

// ---------------------------------------------------------------------------
// Return-map network, finishing pass: apply the network's stress increment
// and dR to each queued particle (dR kept non-negative, as the hardening law
// gives), with the plastic strain increment recovered as de - C^-1 dsigma
// (the compliance of …_VonMisesHardening.cpp:64-71), and re-check a hashed
// fraction of the particles against the exact map computed in FP64 on the
// same inputs (cr_increment_wide; the network's error is recorded; then a
// guard replaces implausible results by that exact map, see below;
// the network's result is kept).
// ---------------------------------------------------------------------------
static __global__ void k_sg_finish(PView<float> P, SurrogateQueue q, MatConst M, int contact, double dt, double inv_yield,
                            float recheck, unsigned long long step, const unsigned long long* step_dev,
                            SurrogateAcc* acc, SurrogateGuard gd) {
    if (step_dev) step = *step_dev;
    const unsigned cnt = (unsigned)min((unsigned long long)*q.count, (unsigned long long)q.cap);
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&acc->queued, (unsigned long long)cnt);
    const unsigned thr = (unsigned)(recheck * 4294967296.0f);
    for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < cnt; s += gridDim.x * blockDim.x) {
        const long long p = q.pidx[s];
        const float* qi = q.in + (long long)s * 13;
        const float* qo = q.out + (long long)s * 7;
        float sig[6], e[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            sig[k] = qi[k];
            e[k] = qi[7 + k];
        }
        const float R = qi[6];
        CrOut<float> o;
#pragma unroll
        for (int k = 0; k < 6; ++k) o.dsig[k] = qo[k];
        o.dR = fmaxf(qo[6], 0.0f);
        const float iE = M.finv_E, nE = M.fnu_over_E, iG = M.finv_G;
        o.deps_p[0] = e[0] - (o.dsig[0] * iE - o.dsig[1] * nE - o.dsig[2] * nE);
        o.deps_p[1] = e[1] - (o.dsig[1] * iE - o.dsig[0] * nE - o.dsig[2] * nE);
        o.deps_p[2] = e[2] - (o.dsig[2] * iE - o.dsig[0] * nE - o.dsig[1] * nE);
        o.deps_p[3] = e[3] - o.dsig[3] * iG;
        o.deps_p[4] = e[4] - o.dsig[4] * iG;
        o.deps_p[5] = e[5] - o.dsig[5] * iG;
        // recheck: a hash of (step, particle) below the fraction
        unsigned long long h = (step + 1) * 0x9e3779b97f4a7c15ULL ^ ((unsigned long long)p * 0xbf58476d1ce4e5b9ULL);
        h = (h ^ (h >> 31)) * 0x94d049bb133111ebULL;
        if ((unsigned)(h >> 32) < thr) {
            // the judge: the exact map in FP64 on the same inputs
            CrOut<double> x;
            cr_increment_wide(M, R, sig, e, x);
            double sq = 0.0, mx = 0.0;
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                const double d = fabs(fps_f2d(o.dsig[k]) - x.dsig[k]) * inv_yield;
                sq += d * d;
                mx = fmax(mx, d);
            }
            atomicAdd(&acc->rechecked, 1ULL);
            atomicAdd(&acc->sq_err, sq / 6.0);
            atomicMax(reinterpret_cast<unsigned long long*>(&acc->max_err), (unsigned long long)__double_as_longlong(mx));
        }
        // the guard: an input outside the training box, or a result that is not the radial return of its trial
        // state (the new stress off the yield surface k0 + R/sqrt 2, a correction dsigma - D de with a
        // hydrostatic part, or a stress or R increment that differs from the radial return evaluated here in
        // FP32; each by more than tol k0), takes the exact map in FP64 instead
        if (gd.tol > 0.0f) {
            bool ok = true;
#pragma unroll
            for (int c = 0; c < 13; ++c) {
                const float xn = qi[c] * gd.in_inv_scale[c];
                ok = ok && xn >= gd.lo[c] && xn <= gd.hi[c];
            }
            float d[6], sn[6];
            trial_increment<float>(M, e, d);
#pragma unroll
            for (int k = 0; k < 6; ++k) sn[k] = sig[k] + o.dsig[k];
            const float a01 = sn[0] - sn[1], a12 = sn[1] - sn[2], a20 = sn[2] - sn[0];
            const float J2 = (a01 * a01 + a12 * a12 + a20 * a20) * (1.0f / 6.0f) + sn[3] * sn[3] + sn[4] * sn[4] +
                             sn[5] * sn[5];
            const float rad = M.fk0 + R * 0.70710678118654752440f;
            const float hyd = ((o.dsig[0] - d[0]) + (o.dsig[1] - d[1]) + (o.dsig[2] - d[2])) * (1.0f / 3.0f);
            const float lim = gd.tol * M.fk0;
            ok = ok && fabsf(sqrtf(J2) - rad) <= lim && fabsf(hyd) <= lim;
            if (ok) {
                // the direction and the hardening: against the FP32 radial return of the same trial state
                CrTrial<float> tr;
                cr_trial<float>(M, R, sig, e, tr);
                CrOut<float> x;
                cr_return<float>(M, R, sig, e, tr, x);
#pragma unroll
                for (int k = 0; k < 6; ++k) ok = ok && fabsf(o.dsig[k] - x.dsig[k]) <= lim;
                ok = ok && fabsf(o.dR - x.dR) <= lim;
            }
            if (!ok) {
                CrOut<double> w;
                cr_increment_wide(M, R, sig, e, w);
                cr_narrow(w, o);
                atomicAdd(&acc->rejected, 1ULL);
            }
        }
        apply_increment<float>(P, p, sig, e, o, q.vol[s], R, contact, dt);
    }
}

}  // namespace mpm
