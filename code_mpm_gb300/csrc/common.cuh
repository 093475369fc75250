// Shared device-side types of the GB300 MPM engine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fpsplit.h"

namespace mpm {

constexpr unsigned FULL_MASK = 0xffffffffu;

// Bits of the sticky device error word.
constexpr unsigned ERR_NONFINITE_POSITION = 1u;
constexpr unsigned ERR_BAD_MATERIAL = 2u;
constexpr unsigned ERR_WAIT_TIMEOUT = 4u;  // a kernel's bounded wait on an mbarrier ran out

// Internal particle flag: member of the displacement-control list.
constexpr unsigned PF_IN_DC = 32u;

// Grid geometry of one specimen.  A context holds one or more specimens,
// each with its own regular grid (GridPoint_Factory::createGrid,
// GridPoint_Factory.h:33-68); their nodes and cell keys are numbered one
// after the other (node_off, key_off).  Kernels receive specimen 0's record
// by value; with several specimens, `tab` holds every record in device
// memory and a particle's record is tab[specimen id].  Node coordinates come
// from the padded per-axis tables xtab (axis a at xtab + xoff[a], entry n+1
// for node index n in [-1, nn[a]]), each computed as (i*L)/cells like
// createGrid (GridPoint_Factory.h:53-55).
struct Geom {
    double h[3];      // cell size = length/cells (GridPoint_Mediator d3_Length_Cell)
    double inv_h[3];  // RN(1/h)
    float hf[3];      // RN32(h)
    float inv_hf[3];  // RN32(inv_h)
    float ih_lo[3];   // RN32(inv_h - inv_hf): inv_hf + ih_lo is inv_h to 2^-48
    int nn[3];        // nodes per axis = cells + 1
    int kd[3];        // cell-key extents = cells + 2 (base cells -1..cells)
    unsigned key_max; // total key count over all specimens: the key of a particle with no node in range
    long long n_nodes;  // total node count over all specimens
    const double* xtab;
    int xoff[3];
    unsigned key_off;    // this specimen's first cell key
    long long node_off;  // this specimen's first node index
    const struct Geom* tab;  // all specimens (device), or null with one specimen
    int nspec;
};

// Float images of a specimen's cell size (set on the host after h, inv_h).
inline void set_float_geometry(Geom& g, int a) {
    g.hf[a] = (float)g.h[a];
    g.inv_hf[a] = (float)g.inv_h[a];
    g.ih_lo[a] = (float)(g.inv_h[a] - (double)g.inv_hf[a]);
}

// The geometry of particle p's specimen.
__device__ __forceinline__ const Geom& spec_geom(const Geom& g, const uint16_t* __restrict__ sid, long long p) {
    return (g.nspec > 1) ? g.tab[sid[p]] : g;
}

// Decode a cell key into the base (bottom-left-far) cell index of its specimen.
__device__ __forceinline__ void key_to_base(unsigned key, const Geom& g, int b[3]) {
    unsigned k = key - g.key_off;
    b[0] = (int)(k % (unsigned)g.kd[0]) - 1;
    k /= (unsigned)g.kd[0];
    b[1] = (int)(k % (unsigned)g.kd[1]) - 1;
    b[2] = (int)(k / (unsigned)g.kd[1]) - 1;
}

__device__ __forceinline__ double node_coord(const Geom& g, int a, int n) { return g.xtab[g.xoff[a] + n + 1]; }

// Node index of corner k (k = 4*ix + 2*iy + iz, the loop order of
// findAdjacentGridPoints, GridPoint_Mediator.cpp:30-50); -1 when out of range.
__device__ __forceinline__ long long corner_node(const Geom& g, const int b[3], int k) {
    int nx = b[0] + ((k >> 2) & 1), ny = b[1] + ((k >> 1) & 1), nz = b[2] + (k & 1);
    if (nx < 0 || ny < 0 || nz < 0 || nx > g.nn[0] - 1 || ny > g.nn[1] - 1 || nz > g.nn[2] - 1) return -1;
    return g.node_off + (long long)nx + (long long)ny * g.nn[0] + (long long)nz * g.nn[0] * g.nn[1];
}

// A cell's corner nodes in a form the cell-run kernels stage per slot:
// corner k = 4 ix + 2 iy + iz is node n0 + ix + iy sy + iz sz, in range when
// bit k of mask is set (the same nodes corner_node gives).
struct CellNodes {
    long long n0, sz;
    int sy;
    unsigned mask;
};

__device__ __forceinline__ CellNodes cell_nodes(const Geom& g, const int b[3]) {
    CellNodes c;
    c.sy = g.nn[0];
    c.sz = (long long)g.nn[0] * g.nn[1];
    c.n0 = g.node_off + (long long)b[0] + (long long)b[1] * c.sy + (long long)b[2] * c.sz;
    c.mask = 0u;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int nx = b[0] + ((k >> 2) & 1), ny = b[1] + ((k >> 1) & 1), nz = b[2] + (k & 1);
        if (nx >= 0 && ny >= 0 && nz >= 0 && nx <= g.nn[0] - 1 && ny <= g.nn[1] - 1 && nz <= g.nn[2] - 1)
            c.mask |= 1u << k;
    }
    return c;
}

// corner k's node (in range: bit k of c.mask)
__device__ __forceinline__ long long cell_node(const CellNodes& c, int k) {
    return c.n0 + ((k >> 2) & 1) + (long long)(((k >> 1) & 1) * c.sy) + ((k & 1) ? c.sz : 0ll);
}

// Specimen owning global node i (binary search over the node offsets).
__device__ __forceinline__ const Geom& node_geom(const Geom& g, long long i) {
    if (g.nspec <= 1) return g;
    int lo = 0, hi = g.nspec - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (g.tab[mid].node_off <= i)
            lo = mid;
        else
            hi = mid - 1;
    }
    return g.tab[lo];
}

// Material constants, precomputed on the host with the reference's own
// expressions so that they are bit-identical to the per-call values of
// ConstitutiveRelation_calculateIncrement_*.cpp.
struct MatConst {
    int type;
    int pad;
    double E, nu, Y, C0, C1;
    double C;      // E/(1+nu)/(1-2nu)
    double one_m_nu, half_m_nu;
    double G;      // 0.5*E/(1+nu)
    double k0;     // Y/sqrt(3)
    double s23C1;  // sqrt(2/3)*C1
    double inv_E, nu_over_E, inv_G;
    // RN32 images of the constants the FP32 form uses
    float fC, fone_m_nu, fnu, fhalf_m_nu, fk0, fs23C1, fC0, finv_E, fnu_over_E, finv_G;
};

inline void set_float_constants(MatConst& k) {
    k.fC = (float)k.C;
    k.fone_m_nu = (float)k.one_m_nu;
    k.fnu = (float)k.nu;
    k.fhalf_m_nu = (float)k.half_m_nu;
    k.fk0 = (float)k.k0;
    k.fs23C1 = (float)k.s23C1;
    k.fC0 = (float)k.C0;
    k.finv_E = (float)k.inv_E;
    k.fnu_over_E = (float)k.nu_over_E;
    k.finv_G = (float)k.inv_G;
}

// An increment of the form's type as a double (exact in both forms).
__device__ __forceinline__ double fps_f2d_form(double v) { return v; }
__device__ __forceinline__ double fps_f2d_form(float v) { return fps_f2d(v); }

// The form's copy of a constant: the double itself, or its float image.
template <typename T>
__device__ __forceinline__ T form_const(double d, float f);
template <>
__device__ __forceinline__ double form_const<double>(double d, float) { return d; }
template <>
__device__ __forceinline__ float form_const<float>(double, float f) { return f; }

// Particle arrays: structure of arrays, component a of particle p at [a*n + p].
template <typename T>
struct PView {
    double* pos;
    T* vel;
    T* fext;
    T* mass;
    T* vol;
    T* vol0;
    T* F;
    T* stress;
    T* strain;
    T* eps_p;
    double* e_strain;
    double* e_strain_max;
    double* e_strain_ti;
    double* e_plastic;
    T* backstress;
    T* mp_mg;  // particle mass gradient (contact path), the form's type
    T* strain_rate;
    int32_t* material;
    uint8_t* pflags;
    float* dc_mult;
    float* loc;  // FP32 form: cell-local coordinate (x - X_b)/h of the current base cell, 3 x n
    const uint16_t* sid;  // specimen of each particle (null with one specimen)
    const unsigned* orig; // FP32 form in cell order: the caller's index of each slot (null: slot = index)
    double* Fe;           // FP64 form: elastic deformation gradient, 9 x n (large-strain pass 2)
    long long n;
};

// Node arrays: structure of arrays, component a of node i at [a*nn + i].
template <typename T>
struct NView {
    T* acc;            // per node 8 values {m, p[3], f[3], 0}: the accumulated mass, momentum and force
                       // interleaved, so one node's are one or two aligned vectors (P2G adds them as such)
    T* vel;
    T* ftemp;
    T* mg;             // mass gradient (contact path), the form's type
    unsigned* state;   // MPM_NS_* bits
    uint8_t* fixed;
    double* friction;
    T* rec;            // scratch: per node 8 values {r, has, v, 0}: r = f/m before pass 1, p/m before
                       // pass 2; has = 1 when m > mass_min; v = node velocity (pass 2 only)
    T* q;              // scratch: remap accumulator sum N m_p v_p, 4 values per node {q[3], 0}
    unsigned* owner;   // scratch: displacement-control last-writer claims, 3 x nn
    unsigned* nowner;  // scratch: contact-normal last-writer claims, nn
    const unsigned* alist;   // active nodes of this step (null: sweep every node)
    const unsigned* acount;  // their number (device)
    long long nn;
};

// Four values loaded or stored as one aligned vector.
template <typename T>
struct alignas(4 * sizeof(T)) Quad {
    T x, y, z, w;
};

// Adds to node i's remap accumulator {q[3], 0}: one vector atomic in FP32.
template <typename T>
__device__ __forceinline__ void q_add(T* q, long long i, T q0, T q1, T q2) {
    T* a = q + 4 * i;
    if constexpr (sizeof(T) == 4) {
        atomicAdd(reinterpret_cast<float4*>(a), make_float4(q0, q1, q2, 0.0f));
    } else {
        atomicAdd(a, q0);
        atomicAdd(a + 1, q1);
        atomicAdd(a + 2, q2);
    }
}

// Adds a contribution to node i's accumulator record: two vector atomics in
// FP32 (one sector), seven scalar ones in FP64.
template <typename T>
__device__ __forceinline__ void acc_add(T* acc, long long i, T m, T p0, T p1, T p2, T f0, T f1, T f2) {
    T* a = acc + 8 * i;
    if constexpr (sizeof(T) == 4) {
        atomicAdd(reinterpret_cast<float4*>(a), make_float4(m, p0, p1, p2));
        atomicAdd(reinterpret_cast<float4*>(a + 4), make_float4(f0, f1, f2, 0.0f));
    } else {
        atomicAdd(a, m);
        atomicAdd(a + 1, p0);
        atomicAdd(a + 2, p1);
        atomicAdd(a + 3, p2);
        atomicAdd(a + 4, f0);
        atomicAdd(a + 5, f1);
        atomicAdd(a + 6, f2);
    }
}

template <typename T>
__device__ __forceinline__ Quad<T> ld_quad(const T* __restrict__ p) {
    return *reinterpret_cast<const Quad<T>*>(p);
}

// Both halves of a node record, a = p[0..3], b = p[4..7]: one 32-byte load in
// FP32 (records are 32-byte aligned and not written while they are read),
// two 32-byte loads in FP64.
template <typename T>
__device__ __forceinline__ void ld_record(const T* __restrict__ p, Quad<T>& a, Quad<T>& b) {
    if constexpr (sizeof(T) == 4) {
        asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
            : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
            : "l"(p));
    } else {
        a = ld_quad(p);
        b = ld_quad(p + 4);
    }
}

// The nodes a node kernel works on, grid-stride: the active-node list when
// one is given, else every node.  The body may `continue`, not `return`.
// Node state bits beside the caller's (1 active, 2 contact, 4 / 8 contact
// flags): a displacement-control claim is set on the node (internal, cleared
// with the claims in the same step).
constexpr unsigned NODE_CLAIMED = 16u;

// As NODE_LOOP, with each thread's next list entry loaded one iteration
// early, so an iteration waits for one memory round trip instead of two.
#define NODE_LOOP_AHEAD(nd, i)                                                                                    \
    for (long long t_ = blockIdx.x * (long long)blockDim.x + threadIdx.x, s_ = (long long)gridDim.x * blockDim.x, \
                   n_ = (nd).alist ? (long long)*(nd).acount : (nd).nn,                                           \
                   next_ = t_ < n_ ? ((nd).alist ? (long long)(nd).alist[t_] : t_) : 0;                           \
         t_ < n_; t_ += s_)                                                                                       \
        if (const long long i = next_; true)                                                                      \
            if (next_ = (t_ + s_ < n_) ? ((nd).alist ? (long long)(nd).alist[t_ + s_] : t_ + s_) : 0; true)

#define NODE_LOOP(nd, i)                                                                        \
    for (long long t_ = blockIdx.x * (long long)blockDim.x + threadIdx.x,                        \
                   n_ = (nd).alist ? (long long)*(nd).acount : (nd).nn;                         \
         t_ < n_; t_ += (long long)gridDim.x * blockDim.x)                                      \
        if (const long long i = (nd).alist ? (long long)(nd).alist[t_] : t_; true)

}  // namespace mpm
