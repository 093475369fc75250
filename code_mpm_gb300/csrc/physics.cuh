// Per-particle physics shared by the step kernels: trilinear bases and the
// constitutive increments.
#pragma once

#include "common.cuh"

namespace mpm {

// ---------------------------------------------------------------------------
// Trilinear (tent) bases of calculateBases_Classic (GridPoint_Mediator.cpp:95-144)
// for the two nodes b and b+1 along one axis.  N = 1 - |d/h| clamped to
// [0,1]; the gradient factor is sign(d)/h when 1e-12 < |d/h| < 1 - 1e-12,
// else 0.  Here d/h is formed as d * (1/h): within a few ulp of the
// reference, which the parity tolerance covers.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void axis_bases(const Geom& g, int a, double x, int b, T N[2], T gf[2]) {
#pragma unroll
    for (int o = 0; o < 2; ++o) {
        double d = x - node_coord(g, a, b + o);
        T r = (T)(d * g.inv_h[a]);
        T ar = r >= (T)0 ? r : -r;
        T nv = (T)1 - ar;
        if (nv < (T)0 || nv > (T)1) nv = (T)0;
        N[o] = nv;
        T s = (T)((d > 0.0) - (d < 0.0));
        gf[o] = (ar > (T)1.0e-12 && ar < (T)(1.0 - 1.0e-12)) ? s * (T)g.inv_h[a] : (T)0;
    }
}

// FP32 (chosen) form: one FP64 subtraction and product per axis give the
// cell-local coordinate u = (x - X_b)/h in [0, 1); both nodes' bases follow
// in FP32 (d/h = u and u - 1).  FP64 instructions cost ~60 FP32 ones on this
// part, so the chosen form keeps them to this one pair per axis.
__device__ __forceinline__ void axis_bases_local(const Geom& g, int a, double x, int b, float N[2], float gf[2]) {
    const float u = (float)((x - node_coord(g, a, b)) * g.inv_h[a]);
    const float r[2] = {u, u - 1.0f};
    const float ih = (float)g.inv_h[a];
#pragma unroll
    for (int o = 0; o < 2; ++o) {
        float ar = fabsf(r[o]);
        float nv = 1.0f - ar;
        if (nv < 0.0f || nv > 1.0f) nv = 0.0f;
        N[o] = nv;
        float s = (float)((r[o] > 0.0f) - (r[o] < 0.0f));
        gf[o] = (ar > 1.0e-12f && ar < (float)(1.0 - 1.0e-12)) ? s * ih : 0.0f;
    }
}

// FP32 form, from the stored cell-local coordinate u (no FP64 at all).  The
// general form per node offset o is r = u - o, N = 1 - |r| (0 outside
// [0, 1]), gradient sign(r) ih where 1e-12 < |r| < 1; every stored u lies in
// [0, 1] (a fraction minus its floor, or the split form's (1e-4, 1 - 1e-4)),
// where that reduces to the lines below, value for value.
__device__ __forceinline__ void axis_bases_u(float u, float ih, float N[2], float gf[2]) {
    const float a1 = fabsf(u - 1.0f);
    N[0] = 1.0f - u;
    N[1] = 1.0f - a1;
    gf[0] = (u > 1.0e-12f && u < 1.0f) ? ih : 0.0f;
    gf[1] = (a1 > 1.0e-12f && a1 < 1.0f) ? -ih : 0.0f;
}

template <typename T>
struct Bases {
    T Nx[2], Ny[2], Nz[2];
    T gx[2], gy[2], gz[2];
    __device__ __forceinline__ void init(const Geom& g, const double x[3], const int b[3]) {
        if constexpr (sizeof(T) == 4) {
            axis_bases_local(g, 0, x[0], b[0], Nx, gx);
            axis_bases_local(g, 1, x[1], b[1], Ny, gy);
            axis_bases_local(g, 2, x[2], b[2], Nz, gz);
        } else {
            axis_bases<T>(g, 0, x[0], b[0], Nx, gx);
            axis_bases<T>(g, 1, x[1], b[1], Ny, gy);
            axis_bases<T>(g, 2, x[2], b[2], Nz, gz);
        }
    }
    // FP32 form: bases from the cell-local coordinate stored by the previous step
    __device__ __forceinline__ void init_local(const Geom& g, const float u[3]) {
        axis_bases_u(u[0], g.inv_hf[0], (float*)Nx, (float*)gx);
        axis_bases_u(u[1], g.inv_hf[1], (float*)Ny, (float*)gy);
        axis_bases_u(u[2], g.inv_hf[2], (float*)Nz, (float*)gz);
    }
    // corner k = 4*ix + 2*iy + iz (selects, not indexing, so the bases stay
    // in registers when k is a loop variable)
    __device__ __forceinline__ void corner(int k, T& N, T G[3]) const {
        const bool ix = (k >> 2) & 1, iy = (k >> 1) & 1, iz = k & 1;
        const T nx = ix ? Nx[1] : Nx[0], ny = iy ? Ny[1] : Ny[0], nz = iz ? Nz[1] : Nz[0];
        N = nx * ny * nz;
        G[0] = -(ny * nz) * (ix ? gx[1] : gx[0]);
        G[1] = -(nx * nz) * (iy ? gy[1] : gy[0]);
        G[2] = -(nx * ny) * (iz ? gz[1] : gz[0]);
    }
};

// ---------------------------------------------------------------------------
// Correctly rounded quotient a/b given y = RN(1/b): q = RN(a*y),
// r = fma(-q, b, a) (exact), q' = fma(r, y, q) -- Markstein's correction
// step (IBM J. Res. Dev. 34(1), 1990).  Equal to IEEE a/b on the operands
// divided here (checked bit for bit by oracle/div_check.c), at 3 FP64
// operations instead of a full division.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double div_rn_by(double a, double b, double y) {
    double q = __dmul_rn(a, y);
    double r = __fma_rn(-q, b, a);
    return __fma_rn(r, y, q);
}

// ---------------------------------------------------------------------------
// Base cell b = floor(x/h) along axis a, bit-identical to the floor of the
// correctly rounded quotient (GridPoint_Mediator.cpp:8), and the cell-local
// coordinate u = x/h - b as a float.  Fast path: q = RN(x * RN(1/h)) is
// within 2.3e-16 |q| of x/h and RN(x/h) within 1.2e-16 |q|; if q's float
// image sits more than 2e-4 from an integer and |q| < 1024 (float half-ulp
// <= 6.1e-5 there), no rounded quotient can cross an integer, so
// floor(q) = floor(RN(x/h)).  Otherwise the corrected quotient decides.
// Returns false for a non-finite quotient.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool cell_and_local(const Geom& g, int a, double x, double& f, float& u) {
    const double q = __dmul_rn(x, g.inv_h[a]);
    const float qf = (float)q;
    const float ff = floorf(qf);
    const float frf = qf - ff;
    if (frf > 2.0e-4f && frf < 1.0f - 2.0e-4f && fabsf(qf) < 1024.0f) {
        f = (double)ff;
        u = (float)(q - f);
        return true;
    }
    const double qe = div_rn_by(x, g.h[a], g.inv_h[a]);
    if (!isfinite(qe)) {
        f = 0.0;
        u = 0.0f;
        return false;
    }
    f = floor(qe);
    u = (float)(qe - f);
    return true;
}

// ---------------------------------------------------------------------------
// Bit-exact restatement of calculateBases_Classic's gradient for one
// (particle, node) pair, used where results must match the reference to the
// bit (contact mass gradients): correctly rounded d/h and the reference's
// association order, with the _rn intrinsics so nothing is contracted.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void exact_gradient(const Geom& g, const double x[3], const int node[3], double G[3]) {
    double Nv[3], d[3], r[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        d[a] = __dadd_rn(x[a], -node_coord(g, a, node[a]));
        r[a] = div_rn_by(d[a], g.h[a], g.inv_h[a]);
        double ar = r[a] >= 0.0 ? r[a] : -r[a];
        Nv[a] = __dadd_rn(1.0, -ar);
        if (Nv[a] < 0.0 || Nv[a] > 1.0) Nv[a] = 0.0;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        double ar = r[a] >= 0.0 ? r[a] : -r[a];
        G[a] = 0.0;
        if (ar > 1.0e-12 && ar < 1.0 - 1.0e-12) {
            double o1 = Nv[a == 0 ? 1 : 0], o2 = Nv[a == 2 ? 1 : 2];
            double sg = (double)((d[a] > 0.0) - (d[a] < 0.0));
            G[a] = div_rn_by(__dmul_rn(__dmul_rn(-o1, o2), sg), g.h[a], g.inv_h[a]);
        }
    }
}

// glm::dot / glm::length without contraction (glmshim order: (x*x + y*y) + z*z).
__device__ __forceinline__ double dot3_rn(const double a[3], const double b[3]) {
    return __dadd_rn(__dadd_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])), __dmul_rn(a[2], b[2]));
}
__device__ __forceinline__ double len3_rn(const double a[3]) { return __dsqrt_rn(dot3_rn(a, a)); }

// ---------------------------------------------------------------------------
// Deformation-gradient update and strain increment, per form.
//
// FP64 (plain) form, the reference's arithmetic: diagonal strain increment
// (1 + L_ii dt) - 1 (…MPLocks.cpp:206-219); non-contact F <- F (I + L dt)
// (:242); contact F <- F + (L F) dt (…_Contact.cpp:464); V = det(F) V0 with
// glm's cofactor determinant.
//
// FP32 (chosen) form: the same mathematics rearranged so FP32 keeps the
// small increments: the diagonal strain increment is L_ii dt itself (the
// reference's 1 + x - 1 cancels to noise in FP32), and the stored state is
// H = F - I, updated as H + L dt + H (L dt) (non-contact) or
// H + L dt + (L dt) H (contact), with det(I + H) = 1 + I1 + I2 + I3 of H.
// ---------------------------------------------------------------------------
template <typename T>
struct Kinematics;

template <>
struct Kinematics<double> {
    static __device__ __forceinline__ double strain_diag(double x) { return __dadd_rn(__dadd_rn(1.0, x), -1.0); }
    static __device__ __forceinline__ void update(bool contact, const double F[9], const double L[9],
                                                  const double Ldt[9], double dt, double Fn[9]) {
        if (!contact) {
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    double d0 = (c == 0 ? 1.0 : 0.0) + Ldt[3 * c + 0];
                    double d1 = (c == 1 ? 1.0 : 0.0) + Ldt[3 * c + 1];
                    double d2 = (c == 2 ? 1.0 : 0.0) + Ldt[3 * c + 2];
                    Fn[3 * c + r] = F[r] * d0 + F[3 + r] * d1 + F[6 + r] * d2;
                }
        } else {
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
                for (int r = 0; r < 3; ++r)
                    Fn[3 * c + r] =
                        F[3 * c + r] + (L[r] * F[3 * c] + L[3 + r] * F[3 * c + 1] + L[6 + r] * F[3 * c + 2]) * dt;
        }
    }
    static __device__ __forceinline__ double det(const double m[9]) {
        return m[0] * (m[4] * m[8] - m[7] * m[5]) - m[3] * (m[1] * m[8] - m[7] * m[2]) +
               m[6] * (m[1] * m[5] - m[4] * m[2]);
    }
};

template <>
struct Kinematics<float> {
    static __device__ __forceinline__ float strain_diag(float x) { return x; }
    // H (= F - I) in, Hn out
    static __device__ __forceinline__ void update(bool contact, const float H[9], const float L[9], const float Ldt[9],
                                                  float dt, float Hn[9]) {
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                float prod = contact ? (Ldt[r] * H[3 * c] + Ldt[3 + r] * H[3 * c + 1] + Ldt[6 + r] * H[3 * c + 2])
                                     : (H[r] * Ldt[3 * c] + H[3 + r] * Ldt[3 * c + 1] + H[6 + r] * Ldt[3 * c + 2]);
                Hn[3 * c + r] = H[3 * c + r] + (Ldt[3 * c + r] + prod);
            }
    }
    // det(I + H) - 1 = I1 + I2 + I3 of H; returns det(I + H)
    static __device__ __forceinline__ float det(const float h[9]) {
        float i1 = h[0] + h[4] + h[8];
        float i2 = h[0] * h[4] + h[4] * h[8] + h[0] * h[8] - h[3] * h[1] - h[7] * h[5] - h[6] * h[2];
        float i3 = h[0] * (h[4] * h[8] - h[7] * h[5]) - h[3] * (h[1] * h[8] - h[7] * h[2]) +
                   h[6] * (h[1] * h[5] - h[4] * h[2]);
        return 1.0f + (i1 + (i2 + i3));
    }
};

// ---------------------------------------------------------------------------
// Constitutive increments (ConstitutiveRelation_calculateIncrement_*.cpp)
// ---------------------------------------------------------------------------
template <typename T>
struct CrOut {
    T dsig[6];
    T deps_p[6];
    T dR;
};

template <typename T>
__device__ __forceinline__ void trial_increment(const MatConst& m, const T e[6], T d[6]) {
    const T C = form_const<T>(m.C, m.fC), a = form_const<T>(m.one_m_nu, m.fone_m_nu),
            nu = form_const<T>(m.nu, m.fnu), hb = form_const<T>(m.half_m_nu, m.fhalf_m_nu);
    d[0] = C * (a * e[0] + nu * e[1] + nu * e[2]);
    d[1] = C * (a * e[1] + nu * e[0] + nu * e[2]);
    d[2] = C * (a * e[2] + nu * e[0] + nu * e[1]);
    d[3] = C * (hb * e[3]);
    d[4] = C * (hb * e[4]);
    d[5] = C * (hb * e[5]);
}

// The trial state of a constitutive increment: the elastic predictor
// dtr = D de and, for the plastic laws, the trial stress tr = sig + dtr, its
// J2 and the yield radius rad (k0, plus R/sqrt 2 with hardening).
template <typename T>
struct CrTrial {
    T dtr[6], tr[6];
    T J2, rad;
};

template <typename T>
__device__ __forceinline__ void cr_trial(const MatConst& m, T R, const T sig[6], const T e[6], CrTrial<T>& t) {
    trial_increment<T>(m, e, t.dtr);
    if (m.type == 0) return;
#pragma unroll
    for (int i = 0; i < 6; ++i) t.tr[i] = sig[i] + t.dtr[i];
    const T a01 = t.tr[0] - t.tr[1], a12 = t.tr[1] - t.tr[2], a20 = t.tr[2] - t.tr[0];
    T J2 = (T)(1.0 / 6.0) * a01 * a01;
    J2 += (T)(1.0 / 6.0) * a12 * a12;
    J2 += (T)(1.0 / 6.0) * a20 * a20;
    J2 += t.tr[3] * t.tr[3];
    J2 += t.tr[4] * t.tr[4];
    J2 += t.tr[5] * t.tr[5];
    t.J2 = J2;
    T rad = form_const<T>(m.k0, m.fk0);
    if (m.type == 4) rad = rad + R * (T)0.70710678118654752440;  // R / sqrt(2)
    t.rad = rad;
}

// Elastic (…_Elastic.cpp:4-18); PerfectlyPlastic radial return
// (…_PerfectlyPlastic.cpp:4-76, radius k0); von Mises with explicit
// isotropic hardening (…_VonMisesHardening.cpp:4-92, radius k0 + R/sqrt 2,
// dR = C0 (sqrt(2/3) C1 - R) sqrt(2/3 sum deps_p^2) when positive), from
// the trial state.
template <typename T>
__device__ __forceinline__ void cr_return(const MatConst& m, T R, const T sig[6], const T e[6], const CrTrial<T>& t,
                                          CrOut<T>& o) {
    o.dR = (T)0;
#pragma unroll
    for (int i = 0; i < 6; ++i) o.deps_p[i] = (T)0;
    if (m.type == 0 || t.J2 <= t.rad * t.rad) {
#pragma unroll
        for (int i = 0; i < 6; ++i) o.dsig[i] = t.dtr[i];
        return;
    }
    const T hyd = (T)(1.0 / 3.0) * (t.tr[0] + t.tr[1] + t.tr[2]);
    const T sc = t.rad / sqrt(t.J2);
    T dev[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) dev[i] = t.tr[i];
    dev[0] -= hyd;
    dev[1] -= hyd;
    dev[2] -= hyd;
#pragma unroll
    for (int i = 0; i < 6; ++i) o.dsig[i] = dev[i] * sc - sig[i];
    o.dsig[0] += hyd;
    o.dsig[1] += hyd;
    o.dsig[2] += hyd;
    const T iE = form_const<T>(m.inv_E, m.finv_E), nE = form_const<T>(m.nu_over_E, m.fnu_over_E),
            iG = form_const<T>(m.inv_G, m.finv_G);
    T ee[6];
    ee[0] = o.dsig[0] * iE - o.dsig[1] * nE - o.dsig[2] * nE;
    ee[1] = o.dsig[1] * iE - o.dsig[0] * nE - o.dsig[2] * nE;
    ee[2] = o.dsig[2] * iE - o.dsig[0] * nE - o.dsig[1] * nE;
    ee[3] = o.dsig[3] * iG;
    ee[4] = o.dsig[4] * iG;
    ee[5] = o.dsig[5] * iG;
#pragma unroll
    for (int i = 0; i < 6; ++i) o.deps_p[i] = e[i] - ee[i];
    if (m.type != 4) return;
    T ep = (T)0;
#pragma unroll
    for (int i = 0; i < 6; ++i) ep += o.deps_p[i] * o.deps_p[i];
    ep = sqrt(ep * (T)(2.0 / 3.0));
    const T sat = form_const<T>(m.s23C1, m.fs23C1) - R;
    o.dR = (sat > (T)0) ? form_const<T>(m.C0, m.fC0) * sat * ep : (T)0;
}

template <typename T>
__device__ __forceinline__ void cr_increment(const MatConst& m, T R, const T sig[6], const T e[6], CrOut<T>& o) {
    CrTrial<T> t;
    cr_trial<T>(m, R, sig, e, t);
    cr_return<T>(m, R, sig, e, t, o);
}

// The exact map in FP64 on FP32 state (the chosen form's fallback path and
// the judge of the learned map): the float inputs widened exactly, the
// increment computed in double (cr_increment<double>, the plain form's
// arithmetic), each output rounded once to float.
__device__ __forceinline__ void cr_increment_wide(const MatConst& m, float R, const float sig[6], const float e[6],
                                                  CrOut<double>& w) {
    double s64[6], e64[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        s64[i] = fps_f2d(sig[i]);
        e64[i] = fps_f2d(e[i]);
    }
    cr_increment<double>(m, fps_f2d(R), s64, e64, w);
}

__device__ __forceinline__ void cr_narrow(const CrOut<double>& w, CrOut<float>& o) {
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        o.dsig[i] = __double2float_rn(w.dsig[i]);
        o.deps_p[i] = __double2float_rn(w.deps_p[i]);
    }
    o.dR = __double2float_rn(w.dR);
}

// ---------------------------------------------------------------------------
// Large-strain pass 2 helpers (FP64 form; G2P_P2_LargeStrain,
// PhysicsEngine_runSimulation_Classic_DoublePass_MPLocks.cpp:281-437).  glm
// column-major 3x3 (element [c][r] at 3c + r); the products associate as
// glm's operator*: (A B)[c][r] = A[0][r] B[c][0] + A[1][r] B[c][1] + A[2][r] B[c][2].
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mat3_mul(const double A[9], const double B[9], double R[9]) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) R[3 * c + r] = A[r] * B[3 * c] + A[3 + r] * B[3 * c + 1] + A[6 + r] * B[3 * c + 2];
}

// log A = sum over n = 1..8 of (-1)^(n+1) (A - I)^n / n and exp A = sum over
// n = 0..8 of A^n / n!, the truncated series of getLog / getExp
// (ConstitutiveRelation_MatrixAlgebra.cpp:25-53); each power is the previous
// one times the base, as getPower forms it.
__device__ __forceinline__ void mat3_log8(const double A[9], double R[9]) {
    double B[9], P[9], T[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const double I = (k == 0 || k == 4 || k == 8) ? 1.0 : 0.0;
        B[k] = A[k] - I;
        P[k] = I;
        R[k] = 0.0;
    }
#pragma unroll 1
    for (int n = 1; n <= 8; ++n) {
        mat3_mul(P, B, T);
        const double inv = 1.0 / n, sign = (n & 1) ? 1.0 : -1.0;
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            P[k] = T[k];
            R[k] = R[k] + (P[k] * inv) * sign;
        }
    }
}

__device__ __forceinline__ void mat3_exp8(const double A[9], double R[9]) {
    double P[9], T[9], fact = 1.0;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        P[k] = (k == 0 || k == 4 || k == 8) ? 1.0 : 0.0;
        R[k] = P[k];
    }
#pragma unroll 1
    for (int n = 1; n <= 8; ++n) {
        mat3_mul(P, A, T);
        fact *= n;
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            P[k] = T[k];
            R[k] = R[k] + P[k] / fact;
        }
    }
}

// 0.5 log(M M^T) in Voigt order with engineering shear
__device__ __forceinline__ void half_log_voigt(const double M[9], double v[6]) {
    double Mt[9], MMt[9], lg[9];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) Mt[3 * c + r] = M[3 * r + c];
    mat3_mul(M, Mt, MMt);
    mat3_log8(MMt, lg);
#pragma unroll
    for (int k = 0; k < 9; ++k) lg[k] = 0.5 * lg[k];
    v[0] = lg[0];
    v[1] = lg[4];
    v[2] = lg[8];
    v[3] = lg[1] + lg[3];
    v[4] = lg[5] + lg[7];
    v[5] = lg[6] + lg[2];
}

}  // namespace mpm
