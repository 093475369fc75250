// Shared device-side types of the GB300 MPM engine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mpm {

constexpr unsigned FULL_MASK = 0xffffffffu;

// Bits of the sticky device error word.
constexpr unsigned ERR_NONFINITE_POSITION = 1u;
constexpr unsigned ERR_BAD_MATERIAL = 2u;

// Internal particle flag: member of the displacement-control list.
constexpr unsigned PF_IN_DC = 32u;

// Grid geometry, by value in every kernel.  Node coordinates come from the
// padded per-axis tables xtab (axis a at xtab + xoff[a], entry n+1 for node
// index n in [-1, nn[a]]), each computed as (i*L)/cells like
// GridPoint_Factory::createGrid (GridPoint_Factory.h:53-55).
struct Geom {
    double h[3];      // cell size = length/cells (GridPoint_Mediator d3_Length_Cell)
    double inv_h[3];  // 1/h, used where the result only has to be within tolerance
    int nn[3];        // nodes per axis = cells + 1
    int kd[3];        // cell-key extents = cells + 2 (base cells -1..cells)
    unsigned key_max; // kd0*kd1*kd2: the key of a particle with no grid node in range
    long long n_nodes;
    const double* xtab;
    int xoff[3];
};

// Decode a cell key into the base (bottom-left-far) cell index.
__device__ __forceinline__ void key_to_base(unsigned key, const Geom& g, int b[3]) {
    unsigned k = key;
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
    return (long long)nx + (long long)ny * g.nn[0] + (long long)nz * g.nn[0] * g.nn[1];
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
};

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
    double* mp_mg;
    T* strain_rate;
    int32_t* material;
    uint8_t* pflags;
    float* dc_mult;
    long long n;
};

// Node arrays: structure of arrays, component a of node i at [a*nn + i].
template <typename T>
struct NView {
    T* mass;
    T* mom;
    T* vel;
    T* force;
    T* ftemp;
    double* mg;        // mass gradient (contact path)
    unsigned* state;   // MPM_NS_* bits
    uint8_t* fixed;
    double* friction;
    T* ratio;          // scratch: f/m before pass 1, p/m before pass 2
    T* q;              // scratch: remap accumulator sum N m_p v_p
    unsigned* owner;   // scratch: displacement-control last-writer claims, 3 x nn
    unsigned* nowner;  // scratch: contact-normal last-writer claims, nn
    long long nn;
};

}  // namespace mpm
