// Learned von Mises hardening return map: training samples from the exact
// FP64 map, FP32 training kernels (forward, backward, Adam), and the BF16
// tcgen05 inference kernel.  The network replaces
// ConstitutiveRelation::calculateIncrement_VonMisesHardening
// (ConstitutiveRelation_calculateIncrement_VonMisesHardening.cpp:4-92) for
// clearly plastic trial states; it is this library's addition.
//
// Network: x (13 inputs, padded to 16) -> 128 -> 128 -> 128 (ReLU) -> 8 (7
// used).  ReLU rather than a smooth activation: its inference epilogue is a
// bias add and one packed convert per two values, with nothing on the
// special-function pipe, so the epilogue keeps pace with the tensor core.
// Inputs are scaled to O(1): stress and R by 1/yield, the strain
// increment by 1/deps_sigma; outputs are standardised by the training set's
// mean and standard deviation.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "mpm_surrogate.h"
#include "physics.cuh"
#include "surrogate.cuh"

namespace mpm {
namespace net {

constexpr int IN = 16, NIN = 13, HID = 128, OUT = 8, NOUT = 7;
constexpr long long OW1 = 0, OB1 = OW1 + HID * IN, OW2 = OB1 + HID, OB2 = OW2 + HID * HID, OW3 = OB2 + HID,
                    OB3 = OW3 + HID * HID, OW4 = OB3 + HID, OB4 = OW4 + OUT * HID, NPARAM = OB4 + OUT;

#define NCK(x)                                      \
    do {                                            \
        cudaError_t e_ = (x);                       \
        if (e_ != cudaSuccess) {                    \
            cudaGetLastError();                     \
            return MPM_ERR_CUDA;                    \
        }                                           \
    } while (0)

// ---------------------------------------------------------------------------
// counter-based random numbers (splitmix64 finaliser of (seed, sample, draw))
// ---------------------------------------------------------------------------
__host__ __device__ inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
__device__ inline float uni(uint64_t seed, uint64_t i, uint32_t j) {
    uint64_t h = mix64(seed + 0x9e3779b97f4a7c15ULL * (i * 64 + j + 1));
    return ((float)(h >> 40) + 0.5f) * (1.0f / 16777216.0f);  // (0, 1)
}
__device__ inline float gauss(uint64_t seed, uint64_t i, uint32_t j) {
    float u1 = uni(seed, i, 2 * j + 32), u2 = uni(seed, i, 2 * j + 33);
    return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
}

struct SampleCfg {
    double yield, range, epmax, dsig, C0, C1;
    uint64_t seed;
    int sampling;
};

// One sample: prior stress U(+-range yield), R from the closed form of the
// hardening law for a uniform equivalent plastic strain
// (R = sqrt(2/3) C1 (1 - exp(-C0 epbar)), the solution of dR = C0 (sqrt(2/3)
// C1 - R) depbar), strain increment N(0, dsig); target = the exact FP64
// return map (cr_increment<double>).  x: normalised inputs (16, zero padded),
// raw: physical inputs (13), t: physical outputs (7) and f_trial / k0.
__device__ void label_sample(long long i, const double sig[6], double R, const double e[6], const SampleCfg& sc,
                             const MatConst& M, float* __restrict__ x, float* __restrict__ t);

__global__ void k_generate(long long n, long long i0, SampleCfg sc, MatConst M, float* __restrict__ x,
                           float* __restrict__ t) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t gi = (uint64_t)(i0 + i);
    double sig[6], e[6];
    const double ep = uni(sc.seed, gi, 6) * sc.epmax;
    const double R = sqrt(2.0 / 3.0) * sc.C1 * (1.0 - exp(-sc.C0 * ep));
    if (sc.sampling == 0) {
        for (int c = 0; c < 6; ++c) sig[c] = (2.0 * uni(sc.seed, gi, c) - 1.0) * sc.range * sc.yield;
    } else {
        // a random deviator scaled to sqrt J2 = U(0.85, 1) (k0 + R/sqrt 2), plus a hydrostatic part
        double d[6];
        for (int c = 0; c < 6; ++c) d[c] = gauss(sc.seed, gi, 8 + c);
        const double h = (d[0] + d[1] + d[2]) / 3.0;
        for (int c = 0; c < 3; ++c) d[c] -= h;
        const double j2 = ((d[0] - d[1]) * (d[0] - d[1]) + (d[1] - d[2]) * (d[1] - d[2]) + (d[2] - d[0]) * (d[2] - d[0])) /
                              6.0 + d[3] * d[3] + d[4] * d[4] + d[5] * d[5];
        const double rad = M.k0 + R * 0.70710678118654752440;
        const double sc2 = (0.85 + 0.15 * uni(sc.seed, gi, 7)) * rad / sqrt(j2);
        const double p = (2.0 * uni(sc.seed, gi, 5) - 1.0) * sc.yield;
        for (int c = 0; c < 6; ++c) sig[c] = d[c] * sc2 + (c < 3 ? p : 0.0);
    }
    for (int c = 0; c < 6; ++c) e[c] = gauss(sc.seed, gi, c) * sc.dsig;
    label_sample(i, sig, R, e, sc, M, x, t);
}

// Samples given as physical input rows (e.g. harvested from a run of the
// plain method): labelled by the exact FP64 map like generated ones.
__global__ void k_label_rows(long long n, const float* __restrict__ in, SampleCfg sc, MatConst M,
                             float* __restrict__ x, float* __restrict__ t) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double sig[6], e[6];
    for (int c = 0; c < 6; ++c) {
        sig[c] = in[i * NIN + c];
        e[c] = in[i * NIN + 7 + c];
    }
    label_sample(i, sig, (double)in[i * NIN + 6], e, sc, M, x, t);
}

// normalised inputs x[i] (16) and targets t[i] (plastic correction, dR, f_trial / k0)
__device__ void label_sample(long long i, const double sig[6], double R, const double e[6], const SampleCfg& sc,
                             const MatConst& M, float* __restrict__ x, float* __restrict__ t) {
    CrOut<double> o;
    cr_increment<double>(M, R, sig, e, o);
    // trial yield function (…_VonMisesHardening.cpp:35-46)
    double dtr[6];
    trial_increment<double>(M, e, dtr);
    double tr[6];
    for (int c = 0; c < 6; ++c) tr[c] = sig[c] + dtr[c];
    const double a01 = tr[0] - tr[1], a12 = tr[1] - tr[2], a20 = tr[2] - tr[0];
    const double J2 = (a01 * a01 + a12 * a12 + a20 * a20) / 6.0 + tr[3] * tr[3] + tr[4] * tr[4] + tr[5] * tr[5];
    const double f = sqrt(J2) - (M.k0 + R * 0.70710678118654752440);
    float* xi = x + i * IN;
    for (int c = 0; c < 6; ++c) {
        xi[c] = (float)(sig[c] / sc.yield);
        xi[7 + c] = (float)(e[c] / sc.dsig);
    }
    xi[6] = (float)(R / sc.yield);
    xi[13] = xi[14] = xi[15] = 0.0f;
    // targets: the plastic correction dsigma - D de (the kernels add D de back)
    float* ti = t + i * OUT;
    for (int c = 0; c < 6; ++c) ti[c] = (float)(o.dsig[c] - dtr[c]);
    ti[6] = (float)o.dR;
    ti[7] = (float)(f / M.k0);
}

// Per-column min and max of the normalised inputs x (n x 16, first NIN
// columns) as order-preserving unsigned keys: box[c] min, box[NIN + c] max.
__device__ __forceinline__ unsigned f2ord(float f) {
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void k_box(long long n, const float* __restrict__ x, unsigned* __restrict__ box) {
    unsigned lo[NIN], hi[NIN];
    for (int c = 0; c < NIN; ++c) {
        lo[c] = 0xffffffffu;
        hi[c] = 0u;
    }
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        for (int c = 0; c < NIN; ++c) {
            const unsigned k = f2ord(x[i * IN + c]);
            lo[c] = min(lo[c], k);
            hi[c] = max(hi[c], k);
        }
    for (int c = 0; c < NIN; ++c) {
        const unsigned a = __reduce_min_sync(0xffffffffu, lo[c]), b = __reduce_max_sync(0xffffffffu, hi[c]);
        if ((threadIdx.x & 31) == 0) {
            atomicMin(&box[c], a);
            atomicMax(&box[NIN + c], b);
        }
    }
}

static float ord2f(unsigned k) {
    const unsigned u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    float f;
    memcpy(&f, &u, 4);
    return f;
}

// per-output sums of the targets (mean and standard deviation)
__global__ void k_moments(long long n, const float* __restrict__ t, double* __restrict__ acc) {
    __shared__ double s[2 * NOUT];
    if (threadIdx.x < 2 * NOUT) s[threadIdx.x] = 0.0;
    __syncthreads();
    double a[NOUT] = {}, b[NOUT] = {};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        for (int c = 0; c < NOUT; ++c) {
            double v = t[i * OUT + c];
            a[c] += v;
            b[c] += v * v;
        }
    for (int c = 0; c < NOUT; ++c) {
        atomicAdd(&s[c], a[c]);
        atomicAdd(&s[NOUT + c], b[c]);
    }
    __syncthreads();
    if (threadIdx.x < 2 * NOUT) atomicAdd(&acc[threadIdx.x], s[threadIdx.x]);
}

__global__ void k_normalise_targets(long long n, const float* __restrict__ t, const float* __restrict__ shift,
                                    const float* __restrict__ inv_scale, float* __restrict__ tn) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int c = 0; c < NOUT; ++c) tn[i * OUT + c] = (t[i * OUT + c] - shift[c]) * inv_scale[c];
    tn[i * OUT + 7] = 0.0f;
}

// ---------------------------------------------------------------------------
// FP32 GEMM for training: C[M x N] = op(A)[M x K] op(B)[K x N], 64 x 64 tiles,
// 16-deep k slices, 4 x 4 outputs per thread.  op(A) = A (row-major, lda) or
// A^T (A stored K x M); op(B) = B (row-major K x N) or B^T (B stored N x K,
// the layer weights W[out][in]).  Epilogues: store (+bias), bias + ReLU
// (keeps the pre-activation in aux), times ReLU'(aux) (backward), and atomic
// accumulation of split-K partial sums (weight gradients; blockIdx.z picks
// the k range).
// ---------------------------------------------------------------------------
enum { EPI_STORE = 0, EPI_RELU = 1, EPI_DRELU = 2, EPI_ATOMIC = 3 };

template <bool TA, bool TB, int EPI>
__global__ void __launch_bounds__(256) k_sgemm(int M, int N, int K, const float* __restrict__ A, int lda,
                                               const float* __restrict__ B, int ldb, float* __restrict__ C, int ldc,
                                               const float* __restrict__ bias, float* __restrict__ aux, int kchunk) {
    __shared__ __align__(16) float As[16][68];
    __shared__ __align__(16) float Bs[16][68];
    const int tid = threadIdx.x;
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    const int kbeg = blockIdx.z * kchunk, kend = min(K, kbeg + kchunk);
    const int tm = (tid >> 4) * 4, tn = (tid & 15) * 4;
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;
    for (int k0 = kbeg; k0 < kend; k0 += 16) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int e = tid + r * 256;
            int mm, kk;
            if (!TA) {
                mm = e >> 4;
                kk = e & 15;
            } else {
                kk = e >> 6;
                mm = e & 63;
            }
            const int gm = m0 + mm, gk = k0 + kk;
            float v = 0.0f;
            if (gm < M && gk < kend) v = TA ? A[(long long)gk * lda + gm] : A[(long long)gm * lda + gk];
            As[kk][mm] = v;
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int e = tid + r * 256;
            int kk, nn;
            if (!TB) {
                kk = e >> 6;
                nn = e & 63;
            } else {
                nn = e >> 4;
                kk = e & 15;
            }
            const int gn = n0 + nn, gk = k0 + kk;
            float v = 0.0f;
            if (gn < N && gk < kend) v = TB ? B[(long long)gn * ldb + gk] : B[(long long)gk * ldb + gn];
            Bs[kk][nn] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            const float4 a = *reinterpret_cast<const float4*>(&As[kk][tm]);
            const float4 b = *reinterpret_cast<const float4*>(&Bs[kk][tn]);
            const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int m = m0 + tm + i, n = n0 + tn + j;
            if (m >= M || n >= N) continue;
            float v = acc[i][j];
            const long long o = (long long)m * ldc + n;
            if constexpr (EPI == EPI_STORE) {
                if (bias) v += bias[n];
                C[o] = v;
            } else if constexpr (EPI == EPI_RELU) {
                v += bias[n];
                aux[o] = v;
                C[o] = fmaxf(v, 0.0f);
            } else if constexpr (EPI == EPI_DRELU) {
                C[o] = aux[o] > 0.0f ? v : 0.0f;
            } else {
                atomicAdd(&C[o], v);
            }
        }
}

template <bool TA, bool TB, int EPI>
static void sgemm(cudaStream_t s, int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C,
                  int ldc, const float* bias = nullptr, float* aux = nullptr, int splits = 1) {
    const int kchunk = ((K + splits - 1) / splits + 15) / 16 * 16;
    splits = (K + kchunk - 1) / kchunk;
    dim3 grid((N + 63) / 64, (M + 63) / 64, splits);
    k_sgemm<TA, TB, EPI><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, aux, kchunk);
}

// column sums of an n x N row-major matrix into g (atomic; N divides 256)
template <int N>
__global__ void k_colsum(long long n, const float* __restrict__ d, float* __restrict__ g) {
    static_assert(256 % N == 0, "N must divide 256");
    constexpr int RPI = 256 / N;
    const int col = threadIdx.x % N, r0 = threadIdx.x / N;
    const long long base = blockIdx.x * 1024LL;
    float s = 0.0f;
    for (int r = r0; r < 1024; r += RPI) {
        const long long i = base + r;
        if (i < n) s += d[i * N + col];
    }
    atomicAdd(&g[col], s);
}

// loss (mean over samples and the 7 used outputs) and its gradient
__global__ void k_loss(long long n, const float* __restrict__ y, const float* __restrict__ t, float* __restrict__ dy,
                       double* __restrict__ loss) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double l = 0.0;
    if (i < n) {
        const float sc = 2.0f / (float)(n * NOUT);
        for (int c = 0; c < OUT; ++c) {
            const float d = c < NOUT ? y[i * OUT + c] - t[i * OUT + c] : 0.0f;
            dy[i * OUT + c] = sc * d;
            l += (double)d * d;
        }
    }
    for (int o = 16; o; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, l / (double)(n * NOUT));
}

__global__ void k_adam(long long n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// rows of the training set in a pseudo-random order: row j of the epoch is
// (a j + c) mod n with a coprime to n (a full-period affine permutation)
__global__ void k_gather(long long n, const float* __restrict__ x, const float* __restrict__ t, long long a,
                         long long c, long long j0, int rows, float* __restrict__ xb, float* __restrict__ tb) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const unsigned long long j = (unsigned long long)(j0 + r);
    const long long i = (long long)(((unsigned __int128)a * j + (unsigned long long)c) % (unsigned long long)n);
    const float4* xs = reinterpret_cast<const float4*>(x + i * IN);
    float4* xd = reinterpret_cast<float4*>(xb + (long long)r * IN);
#pragma unroll
    for (int k = 0; k < 4; ++k) xd[k] = xs[k];
    const float4* ts = reinterpret_cast<const float4*>(t + i * OUT);
    float4* td = reinterpret_cast<float4*>(tb + (long long)r * OUT);
    td[0] = ts[0];
    td[1] = ts[1];
}

// validation errors in physical units: sums of squared dstress/yield errors
// (all samples, and those outside the fallback band), max outside the band,
// squared dR/yield errors
__global__ void k_val_errors(long long n, const float* __restrict__ yn, const float* __restrict__ t,
                             const float* __restrict__ shift, const float* __restrict__ scale, float inv_yield,
                             float band, double* __restrict__ acc, unsigned* __restrict__ maxbits) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double s_all = 0, s_out = 0, s_r = 0, cnt_out = 0;
    float mx = 0.0f;
    if (i < n) {
        const bool outside = fabsf(t[i * OUT + 7]) >= band;
        for (int c = 0; c < 6; ++c) {
            const float y = yn[i * OUT + c] * scale[c] + shift[c];
            const float d = (y - t[i * OUT + c]) * inv_yield;
            s_all += (double)d * d;
            if (outside) {
                s_out += (double)d * d;
                mx = fmaxf(mx, fabsf(d));
            }
        }
        const float yr = yn[i * OUT + 6] * scale[6] + shift[6];
        const float dr = (yr - t[i * OUT + 6]) * inv_yield;
        s_r = (double)dr * dr;
        cnt_out = outside ? 1.0 : 0.0;
    }
    for (int o = 16; o; o >>= 1) {
        s_all += __shfl_down_sync(0xffffffffu, s_all, o);
        s_out += __shfl_down_sync(0xffffffffu, s_out, o);
        s_r += __shfl_down_sync(0xffffffffu, s_r, o);
        cnt_out += __shfl_down_sync(0xffffffffu, cnt_out, o);
        mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&acc[0], s_all);
        atomicAdd(&acc[1], s_out);
        atomicAdd(&acc[2], s_r);
        atomicAdd(&acc[3], cnt_out);
        atomicMax(maxbits, __float_as_uint(mx));
    }
}

// physical inputs (n x 13) -> normalised rows (n x 16)
__global__ void k_norm_inputs(long long n, const float* __restrict__ in, const float* __restrict__ inv_scale,
                              float* __restrict__ x) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int c = 0; c < NIN; ++c) x[i * IN + c] = in[i * NIN + c] * inv_scale[c];
    x[i * IN + 13] = x[i * IN + 14] = x[i * IN + 15] = 0.0f;
}

// the elastic predictor D de of physical input row `in` (trial_increment, FP32)
__device__ __forceinline__ void elastic_predictor(const MatConst& M, const float* in, float d[6]) {
    float e[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) e[c] = in[7 + c];
    trial_increment<float>(M, e, d);
}

// normalised outputs (n x 8) -> physical (n x 7): correction + D de, dR
__global__ void k_denorm_outputs(long long n, const float* __restrict__ yn, const float* __restrict__ scale,
                                 const float* __restrict__ shift, const float* __restrict__ in, MatConst M,
                                 float* __restrict__ out) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float d[6];
    elastic_predictor(M, in + i * NIN, d);
    for (int c = 0; c < NOUT; ++c) out[i * NOUT + c] = yn[i * OUT + c] * scale[c] + shift[c] + (c < 6 ? d[c] : 0.0f);
}

// the exact return map in FP32 on physical rows: the method without the network
__global__ void k_exact_fp32(long long n, const float* __restrict__ in, MatConst M, float* __restrict__ out) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float sig[6], e[6];
    for (int c = 0; c < 6; ++c) {
        sig[c] = in[i * NIN + c];
        e[c] = in[i * NIN + 7 + c];
    }
    CrOut<float> o;
    cr_increment<float>(M, in[i * NIN + 6], sig, e, o);
    for (int c = 0; c < 6; ++c) out[i * NOUT + c] = o.dsig[c];
    out[i * NOUT + 6] = o.dR;
}

// the exact return map in FP64 on physical rows, outputs rounded once to
// float: the arithmetic of the FP32 form's fallback path (cr_increment_wide)
__global__ void k_exact_wide(long long n, const float* __restrict__ in, MatConst M, float* __restrict__ out) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float sig[6], e[6];
    for (int c = 0; c < 6; ++c) {
        sig[c] = in[i * NIN + c];
        e[c] = in[i * NIN + 7 + c];
    }
    CrOut<double> w;
    cr_increment_wide(M, in[i * NIN + 6], sig, e, w);
    CrOut<float> o;
    cr_narrow(w, o);
    for (int c = 0; c < 6; ++c) out[i * NOUT + c] = o.dsig[c];
    out[i * NOUT + 6] = o.dR;
}

// ---------------------------------------------------------------------------
// BF16 tcgen05 inference (k_mlp_tc, below): tiles of 128 samples; per layer
// one tcgen05.mma (kind::f16, BF16 x BF16 -> FP32, M = 128) per 16 of K with
// the weights (B = W[out][in], N x K) in shared memory, K-major without
// swizzle, and the accumulator D (128 lanes = samples x N columns FP32) in
// tensor memory.  The first layer's A operand (the inputs) is in shared
// memory; the hidden activations are written back to tensor memory
// (tcgen05.st, one lane per sample) and are the A operand of the next layer.
//
// Shared-memory operand layout (K-major, no swizzle): 8-row x 16-byte core
// matrices; element (r, k) of an R-row operand at byte
//   ((k / 8) * (R / 8) + r / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// so core matrices adjacent in K are R/8 * 128 bytes apart (the leading
// byte offset) and 8-row groups 128 bytes apart (the stride byte offset).
// ---------------------------------------------------------------------------
__host__ __device__ constexpr uint32_t kmajor_off(int r, int k, int R) {
    return (uint32_t)(((k >> 3) * (R >> 3) + (r >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor: start address, leading and stride byte
// offsets (>> 4), descriptor version 1 (bits 46-47), no swizzle (bits 61-63 = 0)
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// shared-memory image of the packed weights (bytes).  The hidden layers'
// biases ride in the MMAs: W1's input column 13 holds b1 (the inputs carry a
// 1 there), and W2, W3 have K = 144 with b2, b3 in column 128 (the
// activations carry a 1 in K column 128, zeros up to 143)
constexpr int KH = HID + 16;
constexpr uint32_t SW1 = 0, SW2 = SW1 + HID * IN * 2, SW3 = SW2 + HID * KH * 2, SW4 = SW3 + HID * KH * 2,
                   WBYTES = SW4 + 16 * HID * 2;  // W4 padded to 16 rows
// biases (FP32): b1, b2, b3 (128 each), b4 (16)
constexpr uint32_t NBIAS = 3 * HID + 16;
// kernel shared memory: weights, biases (FP32; the output bias is used), then
// per tile slot (NSLOT) the inputs A0 (128 x 16), the mbarriers (MMA done and
// operand ready per slot, the final drain), the TMEM address.  Tensor memory
// per slot (256 columns): the accumulator D (128 columns) and the hidden
// activations, the A operand of layers 2-4 (128 x 144 BF16 = 72 columns, the
// last 8 the constant bias column), so the MMAs read only the weights from
// shared memory.
constexpr int NSLOT = 2;
constexpr uint32_t SLOT_COLS = 256, TMEM_COLS = SLOT_COLS * NSLOT, ACT_COL = 128;
constexpr uint32_t S_BIAS = WBYTES, S_A0 = (S_BIAS + NBIAS * 4 + 1023) / 1024 * 1024, A0_BYTES = 128 * IN * 2,
                   S_BAR = S_A0 + NSLOT * A0_BYTES, S_TADDR = S_BAR + 8 * (2 * NSLOT + 1),
                   SMEM_TC = S_TADDR + 8 + 1024;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// bounded wait on an mbarrier phase; false (and the error bit) on timeout
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity, unsigned* err) {
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

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// the 64 columns at taddr of this warp's lanes into u: two loads in flight,
// then the wait, in one statement so no use of u precedes the wait
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, uint32_t* u) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,"
        "%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%64];\n"
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,"
        "%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%65];\n"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]),
          "=r"(u[8]), "=r"(u[9]), "=r"(u[10]), "=r"(u[11]), "=r"(u[12]), "=r"(u[13]), "=r"(u[14]), "=r"(u[15]),
          "=r"(u[16]), "=r"(u[17]), "=r"(u[18]), "=r"(u[19]), "=r"(u[20]), "=r"(u[21]), "=r"(u[22]), "=r"(u[23]),
          "=r"(u[24]), "=r"(u[25]), "=r"(u[26]), "=r"(u[27]), "=r"(u[28]), "=r"(u[29]), "=r"(u[30]), "=r"(u[31]),
          "=r"(u[32]), "=r"(u[33]), "=r"(u[34]), "=r"(u[35]), "=r"(u[36]), "=r"(u[37]), "=r"(u[38]), "=r"(u[39]),
          "=r"(u[40]), "=r"(u[41]), "=r"(u[42]), "=r"(u[43]), "=r"(u[44]), "=r"(u[45]), "=r"(u[46]), "=r"(u[47]),
          "=r"(u[48]), "=r"(u[49]), "=r"(u[50]), "=r"(u[51]), "=r"(u[52]), "=r"(u[53]), "=r"(u[54]), "=r"(u[55]),
          "=r"(u[56]), "=r"(u[57]), "=r"(u[58]), "=r"(u[59]), "=r"(u[60]), "=r"(u[61]), "=r"(u[62]), "=r"(u[63])
        : "r"(taddr), "r"(taddr + 32u)
        : "memory");
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}

// 32 words of this warp's lanes to TMEM columns taddr .. taddr + 31 (the
// caller waits with tcgen05.wait::st before the columns are read)
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t* w) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
        "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
        "r"(w[0]), "r"(w[1]), "r"(w[2]), "r"(w[3]), "r"(w[4]), "r"(w[5]), "r"(w[6]), "r"(w[7]), "r"(w[8]), "r"(w[9]),
        "r"(w[10]), "r"(w[11]), "r"(w[12]), "r"(w[13]), "r"(w[14]), "r"(w[15]), "r"(w[16]), "r"(w[17]), "r"(w[18]),
        "r"(w[19]), "r"(w[20]), "r"(w[21]), "r"(w[22]), "r"(w[23]), "r"(w[24]), "r"(w[25]), "r"(w[26]), "r"(w[27]),
        "r"(w[28]), "r"(w[29]), "r"(w[30]), "r"(w[31])
        : "memory");
}

__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t* w) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr), "r"(w[0]),
                 "r"(w[1]), "r"(w[2]), "r"(w[3]), "r"(w[4]), "r"(w[5]), "r"(w[6]), "r"(w[7])
                 : "memory");
}

// D (TMEM) = A (TMEM: 128 lanes = rows, two BF16 of K per 32-bit column) x
// B (shared-memory descriptor), accumulate when acc != 0
__device__ __forceinline__ void mma_bf16_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t b, uint32_t idesc,
                                            uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n" ::"r"(d_tmem),
        "r"(a_tmem), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

// ReLU of two accumulators (their biases already summed in), rounded to BF16
// once: v0 to the low half (element k), v1 to the high half
__device__ __forceinline__ uint32_t relu_bf16x2(float v0, float v1) {
    uint32_t y;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(y) : "f"(v1), "f"(v0));
    return y;
}

// issue one layer: D = A (128 x K) . W^T (W: N x K), K in steps of 16
// (the descriptors of successive K steps differ only in the start address
// field, by two core matrices' leading offsets: one addition each)
// with the activations in tensor memory: K / 16 steps of 8 columns
template <int K, int N>
__device__ __forceinline__ void issue_layer_ts(uint32_t tmem, uint32_t a_tmem, uint32_t w_addr) {
    constexpr uint32_t lbo_b = (uint32_t)(N / 8) * 128;
    constexpr uint32_t id = idesc_bf16(128, N);
    uint64_t b = smem_desc(w_addr, lbo_b, 128);
#pragma unroll
    for (int k = 0; k < K; k += 16) {
        mma_bf16_ts(tmem, a_tmem + (uint32_t)(k / 2), b, id, k > 0 ? 1u : 0u);
        b += (2 * lbo_b) >> 4;
    }
}

template <int K, int N>
__device__ __forceinline__ void issue_layer(uint32_t tmem, uint32_t a_addr, uint32_t w_addr) {
    constexpr uint32_t lbo_a = 128 / 8 * 128, lbo_b = (uint32_t)(N / 8) * 128;
    constexpr uint32_t id = idesc_bf16(128, N);
    uint64_t a = smem_desc(a_addr, lbo_a, 128), b = smem_desc(w_addr, lbo_b, 128);
#pragma unroll
    for (int k = 0; k < K; k += 16) {
        mma_bf16(tmem, a, b, id, k > 0 ? 1u : 0u);
        a += (2 * lbo_a) >> 4;
        b += (2 * lbo_b) >> 4;
    }
}

// hidden-layer epilogue of one tile by its group of WPS warps: thread t of
// group warp j (TMEM lane quarter j % 4) owns sample r = 32 (j % 4) + t and
// columns c0 .. c0 + SPAN - 1; 64 accumulator columns at a time it reads
// them (one wait; the bias is in the sums), applies ReLU and stores the 32
// BF16 pairs to the activation columns (c0 / 2 ...) of its lane
constexpr int WPS = 4;               // epilogue warps per tile slot: 4 (all 128 columns each) or 8 (64 each)
constexpr int SPAN = HID * 4 / WPS;  // columns per epilogue warp

__device__ __forceinline__ void hidden_epilogue(uint32_t d_row, uint32_t act_row, int c0) {
#pragma unroll
    for (int h = c0; h < c0 + SPAN; h += 64) {
        uint32_t u[64], y[32];
        tmem_ld64(d_row + (uint32_t)h, u);
#pragma unroll
        for (int k = 0; k < 32; ++k) y[k] = relu_bf16x2(__uint_as_float(u[2 * k]), __uint_as_float(u[2 * k + 1]));
        tmem_st32(act_row + (uint32_t)(h / 2), y);
    }
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// a sample's 13 physical inputs (zero past n)
__device__ __forceinline__ void load_inputs(const float* __restrict__ in, long long i, long long n, float x[NIN]) {
#pragma unroll
    for (int c = 0; c < NIN; ++c) x[c] = i < n ? in[i * NIN + c] : 0.0f;
}

// a warp's lanes have finished writing an operand: lane 0 arrives on the
// slot's ready barrier (one arrival per warp) once the whole warp's shared
// stores are visible to the tensor core's (async) proxy
__device__ __forceinline__ void warp_arrive_ready(uint32_t bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncwarp();
    if ((threadIdx.x & 31) == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// a warp waits for a barrier phase: lane 0 polls (bounded), the warp follows;
// false on a timeout (same answer in every lane)
__device__ __forceinline__ bool warp_wait(uint32_t bar, uint32_t parity, unsigned* err) {
    int ok = 1;
    if ((threadIdx.x & 31) == 0) ok = bar_wait(bar, parity, err) ? 1 : 0;
    ok = __shfl_sync(FULL_MASK, ok, 0);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    return ok != 0;
}

// non-blocking test of an mbarrier phase
__device__ __forceinline__ bool bar_test(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

struct TcArgs {
    const uint4* wpack;        // WBYTES of packed BF16 weights (the shared-memory image)
    const float* bias;         // NBIAS
    float in_inv_scale[NIN];
    float out_scale[NOUT], out_shift[NOUT];
    const float* in;           // n x 13 physical
    float* out;                // n x 7 physical
    const unsigned* count;     // device sample count (queue), or null
    long long n;               // sample count (or queue capacity)
    unsigned* err;
    MatConst mat;              // for the elastic predictor D de
};

// NSLOT epilogue groups of WPS warps (one per tile slot; warp j of a group
// reads TMEM lane quarter j % 4) and the MMA warp
constexpr int TC_THREADS = 32 * (WPS * NSLOT + 1);

// One CTA per SM takes groups of NSLOT 128-sample tiles, one per slot, and
// runs the slots as independent pipelines that share the tensor core.  A
// slot's epilogue group writes the operand (the inputs into shared memory,
// or the previous layer's activations into tensor memory) and arrives on the
// slot's `ready` mbarrier (one arrival per warp); the MMA warp issues the
// layer of whichever slot is ready and commits to that slot's `full`
// mbarrier; the group waits on `full`, turns the accumulators into the next
// operand, and so on.  The group loads its next tile's inputs while the
// current tile runs.
// Waits are bounded: on a timeout the error word is set and the roles stop;
// the MMA thread then waits (bounded) for its last MMAs before the TMEM is
// freed.
__global__ void __launch_bounds__(TC_THREADS, 1) k_mlp_tc(TcArgs a) {
    extern __shared__ __align__(1024) unsigned char sm[];
    const int t = threadIdx.x, w = t >> 5;
    unsigned char* s = sm + ((1024 - (smem_u32(sm) & 1023u)) & 1023u);  // 1024-byte aligned base
    const uint32_t sbase = smem_u32(s);
    // weights and biases into shared memory (once per CTA)
    for (uint32_t i = t; i < WBYTES / 16; i += TC_THREADS) reinterpret_cast<uint4*>(s)[i] = a.wpack[i];
    float* bias = reinterpret_cast<float*>(s + S_BIAS);
    for (uint32_t i = t; i < NBIAS; i += TC_THREADS) bias[i] = a.bias[i];
    uint32_t* taddr_slot = reinterpret_cast<uint32_t*>(s + S_TADDR);
    // mbarriers: slot sl's MMA-done at full0 + 8 sl, its operand-ready at ready0 + 8 sl
    const uint32_t full0 = sbase + S_BAR, ready0 = full0 + 8 * NSLOT, drain = ready0 + 8 * NSLOT;
    if (t == 0) {
        for (uint32_t sl = 0; sl < NSLOT; ++sl) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(full0 + 8 * sl) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(ready0 + 8 * sl), "n"(WPS) : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(drain) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (w == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(taddr_slot)),
                     "n"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *taddr_slot;
    const long long n = a.count ? (long long)min((unsigned long long)*a.count, (unsigned long long)a.n) : a.n;
    const long long ngroups = (n + 128 * NSLOT - 1) / (128 * NSLOT);
    // tile groups of this CTA: blockIdx.x, blockIdx.x + gridDim.x, ...
    const long long mine = blockIdx.x < ngroups ? (ngroups - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    if (w == WPS * NSLOT) {
        // the MMA warp: lane 0 issues the next layer of any slot whose operand is ready
        if ((t & 31) == 0) {
            const unsigned total = 4u * (unsigned)mine;  // layers per slot
            unsigned issued[NSLOT];
#pragma unroll
            for (int sl = 0; sl < NSLOT; ++sl) issued[sl] = 0u;
            uint32_t ph = 0u;  // bit sl: slot sl's ready parity
            bool ok = true;
            unsigned idle = 0u;
            for (unsigned left = NSLOT * total; left > 0 && ok;) {
                bool progress = false;
#pragma unroll
                for (int sl = 0; sl < NSLOT; ++sl) {
                    if (issued[sl] < total && bar_test(ready0 + 8u * sl, (ph >> sl) & 1u)) {
                        ph ^= 1u << sl;
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        const int layer = (int)(issued[sl] & 3u);
                        const uint32_t d = tmem + SLOT_COLS * sl, act = d + ACT_COL;
                        if (layer == 0)
                            issue_layer<IN, HID>(d, sbase + S_A0 + sl * A0_BYTES, sbase + SW1);
                        else if (layer < 3)
                            issue_layer_ts<KH, HID>(d, act, sbase + (layer == 1 ? SW2 : SW3));
                        else
                            issue_layer_ts<HID, 16>(d, act, sbase + SW4);
                        mma_commit(full0 + 8u * sl);
                        ++issued[sl];
                        --left;
                        progress = true;
                    }
                }
                if (progress) {
                    idle = 0u;
                } else if (++idle > (1u << 26)) {
                    atomicOr(a.err, ERR_WAIT_TIMEOUT);
                    ok = false;
                }
            }
            // every MMA issued has completed before the TMEM is freed
            mma_commit(drain);
            bar_wait(drain, 0u, a.err);
        }
    } else {
        // epilogue group = slot sl; its warp j reads lanes 32 (j % 4) .. + 31, columns c0 .. c0 + SPAN - 1;
        // the warps of columns from 0 own the samples' inputs and outputs
        const int sl = w / WPS, j = w % WPS, r = 32 * (j & 3) + (t & 31), c0 = (j >> 2) * SPAN;
        const bool owner = c0 == 0;
        const uint32_t trow = tmem + SLOT_COLS * (uint32_t)sl + ((uint32_t)(32 * (j & 3)) << 16);
        unsigned char* a0 = s + S_A0 + sl * A0_BYTES;
        if (owner) {
            // the activations' constant K columns 128 .. 143: 1, 0, ..., 0 (the bias column)
            uint32_t one[8] = {0x3F80u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
            tmem_st8(trow + ACT_COL + HID / 2, one);
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        }
        uint32_t ph = 0u;
        bool ok = true;
        float x[NIN];  // the next tile's physical inputs, loaded one tile ahead
        load_inputs(a.in, ((long long)blockIdx.x * NSLOT + sl) * 128 + r, owner ? n : 0, x);
        for (long long k = 0; k < mine && ok; ++k) {
            const long long i = (((long long)blockIdx.x + k * gridDim.x) * NSLOT + sl) * 128 + r;
            // inputs -> A0 (128 x 16 BF16), then the next tile's inputs are requested
            float xn[16];
#pragma unroll
            for (int c = 0; c < 16; ++c) xn[c] = c < NIN ? x[c] * a.in_inv_scale[c] : (c == NIN ? 1.0f : 0.0f);
            float de[6];  // this tile's strain increment, for the elastic predictor
#pragma unroll
            for (int c = 0; c < 6; ++c) de[c] = x[7 + c];
            uint4 p0, p1;
            p0.x = pack_bf16(xn[0], xn[1]);
            p0.y = pack_bf16(xn[2], xn[3]);
            p0.z = pack_bf16(xn[4], xn[5]);
            p0.w = pack_bf16(xn[6], xn[7]);
            p1.x = pack_bf16(xn[8], xn[9]);
            p1.y = pack_bf16(xn[10], xn[11]);
            p1.z = pack_bf16(xn[12], xn[13]);
            p1.w = pack_bf16(xn[14], xn[15]);
            if (owner) {
                *reinterpret_cast<uint4*>(a0 + kmajor_off(r, 0, 128)) = p0;
                *reinterpret_cast<uint4*>(a0 + kmajor_off(r, 8, 128)) = p1;
                load_inputs(a.in, i + (long long)gridDim.x * NSLOT * 128, n, x);
            }
            for (int layer = 0; layer < 4 && ok; ++layer) {
                // the operand (inputs, or the previous layer's activations) is ready
                warp_arrive_ready(ready0 + 8 * sl);
                ok = warp_wait(full0 + 8 * sl, ph, a.err);
                if (!ok) break;
                ph ^= 1u;
                if (layer < 3) {
                    hidden_epilogue(trow, trow + ACT_COL, c0);
                } else if (owner) {
                    float v[16];
                    tmem_ld16(trow, v);
                    if (i < n) {
                        float d[6];
                        trial_increment<float>(a.mat, de, d);  // the elastic predictor D de
#pragma unroll
                        for (int c = 0; c < NOUT; ++c)
                            a.out[i * NOUT + c] =
                                (v[c] + bias[3 * HID + c]) * a.out_scale[c] + a.out_shift[c] + (c < 6 ? d[c] : 0.0f);
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (w == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(TMEM_COLS) : "memory");
}

}  // namespace net
}  // namespace mpm

using namespace mpm;
using namespace mpm::net;

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct mpm_net {
    mpm_net_config cfg;
    MatConst mat;
    int sm_count = 152;
    float* p = nullptr;      // NPARAM master parameters
    float* wpack = nullptr;  // packed BF16 weight image (WBYTES) + biases (NBIAS floats)
    float* scratch = nullptr;
    size_t scratch_bytes = 0;
    unsigned* err = nullptr;
    float in_inv_scale[NIN];
    float out_scale[NOUT], out_shift[NOUT];
    bool packed = false;
    // box of the normalised training inputs (the guard's first check); unbounded until trained
    float box_lo[NIN], box_hi[NIN];
};

static MatConst make_mat(const mpm_net_config& c) {
    MatConst k;
    memset(&k, 0, sizeof(k));
    const double E = c.E, nu = c.nu;
    k.type = 4;
    k.E = E;
    k.nu = nu;
    k.Y = c.yield;
    k.C0 = c.C0;
    k.C1 = c.C1;
    k.C = E / (1.0 + nu) / (1.0 - 2.0 * nu);
    k.one_m_nu = 1.0 - nu;
    k.half_m_nu = 0.5 - nu;
    k.G = 0.5 * E / (1.0 + nu);
    k.k0 = c.yield / std::sqrt(3.0);
    k.s23C1 = std::sqrt(2.0 / 3.0) * c.C1;
    k.inv_E = 1.0 / E;
    k.nu_over_E = nu / E;
    k.inv_G = 1.0 / k.G;
    set_float_constants(k);
    return k;
}

static int ensure_scratch(mpm_net* net, size_t bytes) {
    if (net->scratch_bytes >= bytes) return MPM_OK;
    if (net->scratch) cudaFree(net->scratch);
    net->scratch = nullptr;
    net->scratch_bytes = 0;
    if (cudaMalloc(&net->scratch, bytes) != cudaSuccess) {
        cudaGetLastError();
        return MPM_ERR_NOMEM;
    }
    net->scratch_bytes = bytes;
    return MPM_OK;
}

// BF16 image of the weights in the inference kernel's shared-memory layout
static int pack_weights(mpm_net* net) {
    std::vector<float> p(NPARAM);
    NCK(cudaMemcpy(p.data(), net->p, NPARAM * 4, cudaMemcpyDeviceToHost));
    std::vector<uint16_t> img(WBYTES / 2, 0);
    auto bf = [](float f) -> uint16_t {
        uint32_t u;
        memcpy(&u, &f, 4);
        if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);
        u += 0x7fffu + ((u >> 16) & 1u);
        return (uint16_t)(u >> 16);
    };
    // R x Kimg image of the R x K weights at off, the bias at boff in column kb (kb < 0: none)
    auto put = [&](uint32_t base, int R, int K, int Kimg, long long off, int rows_valid, int kb, long long boff) {
        for (int r = 0; r < R; ++r)
            for (int k = 0; k < Kimg; ++k) {
                float v = 0.0f;
                if (r < rows_valid && k == kb) v = p[boff + r];
                else if (r < rows_valid && k < K) v = p[off + (long long)r * K + k];
                img[(base + kmajor_off(r, k, R)) / 2] = bf(v);
            }
    };
    put(SW1, HID, IN, IN, OW1, HID, NIN, OB1);
    put(SW2, HID, HID, KH, OW2, HID, HID, OB2);
    put(SW3, HID, HID, KH, OW3, HID, HID, OB3);
    put(SW4, 16, HID, HID, OW4, OUT, -1, 0);
    std::vector<float> bias(NBIAS, 0.0f);
    for (int i = 0; i < HID; ++i) {
        bias[i] = p[OB1 + i];
        bias[HID + i] = p[OB2 + i];
        bias[2 * HID + i] = p[OB3 + i];
    }
    for (int i = 0; i < OUT; ++i) bias[3 * HID + i] = p[OB4 + i];
    if (!net->wpack && cudaMalloc(&net->wpack, WBYTES + NBIAS * 4) != cudaSuccess) {
        cudaGetLastError();
        return MPM_ERR_NOMEM;
    }
    NCK(cudaMemcpy(net->wpack, img.data(), WBYTES, cudaMemcpyHostToDevice));
    NCK(cudaMemcpy((char*)net->wpack + WBYTES, bias.data(), NBIAS * 4, cudaMemcpyHostToDevice));
    net->packed = true;
    return MPM_OK;
}

// forward pass on normalised rows x (n x 16) with the FP32 kernels; y (n x 8);
// z1..z3/h1..h3 scratch (n x 128 each)
static void forward_fp32(mpm_net* net, cudaStream_t s, long long n, const float* x, float* z1, float* h1, float* z2,
                         float* h2, float* z3, float* h3, float* y) {
    const float* p = net->p;
    sgemm<false, true, EPI_RELU>(s, (int)n, HID, IN, x, IN, p + OW1, IN, h1, HID, p + OB1, z1);
    sgemm<false, true, EPI_RELU>(s, (int)n, HID, HID, h1, HID, p + OW2, HID, h2, HID, p + OB2, z2);
    sgemm<false, true, EPI_RELU>(s, (int)n, HID, HID, h2, HID, p + OW3, HID, h3, HID, p + OB3, z3);
    sgemm<false, true, EPI_STORE>(s, (int)n, OUT, HID, h3, HID, p + OW4, HID, y, OUT, p + OB4);
}

// gradient of the loss into g (NPARAM, zeroed here); dy already holds dL/dy
static void backward_fp32(mpm_net* net, cudaStream_t s, long long n, const float* x, const float* z1,
                          const float* h1, const float* z2, const float* h2, const float* z3, const float* h3,
                          const float* dy, float* d1, float* d2, float* g) {
    const float* p = net->p;
    cudaMemsetAsync(g, 0, NPARAM * 4, s);
    const int splits = (int)std::max(1LL, std::min(256LL, n / 256));
    const unsigned cb = (unsigned)((n + 1023) / 1024);
    // layer 4
    sgemm<true, false, EPI_ATOMIC>(s, OUT, HID, (int)n, dy, OUT, h3, HID, g + OW4, HID, nullptr, nullptr, splits);
    k_colsum<OUT><<<cb, 256, 0, s>>>(n, dy, g + OB4);
    sgemm<false, false, EPI_DRELU>(s, (int)n, HID, OUT, dy, OUT, p + OW4, HID, d1, HID, nullptr, (float*)z3);
    // layer 3
    sgemm<true, false, EPI_ATOMIC>(s, HID, HID, (int)n, d1, HID, h2, HID, g + OW3, HID, nullptr, nullptr, splits);
    k_colsum<HID><<<cb, 256, 0, s>>>(n, d1, g + OB3);
    sgemm<false, false, EPI_DRELU>(s, (int)n, HID, HID, d1, HID, p + OW3, HID, d2, HID, nullptr, (float*)z2);
    // layer 2
    sgemm<true, false, EPI_ATOMIC>(s, HID, HID, (int)n, d2, HID, h1, HID, g + OW2, HID, nullptr, nullptr, splits);
    k_colsum<HID><<<cb, 256, 0, s>>>(n, d2, g + OB2);
    sgemm<false, false, EPI_DRELU>(s, (int)n, HID, HID, d2, HID, p + OW2, HID, d1, HID, nullptr, (float*)z1);
    // layer 1
    sgemm<true, false, EPI_ATOMIC>(s, HID, IN, (int)n, d1, HID, x, IN, g + OW1, IN, nullptr, nullptr, splits);
    k_colsum<HID><<<cb, 256, 0, s>>>(n, d1, g + OB1);
}

extern "C" {

int64_t mpm_net_param_count(void) { return NPARAM; }

int mpm_net_create(const mpm_net_config* cfg, mpm_net** out) {
    if (!cfg || !out) return MPM_ERR_ARG;
    *out = nullptr;
    if (!(cfg->E > 0) || !(cfg->nu > -1.0 && cfg->nu < 0.5) || !(cfg->yield > 0) || cfg->n_samples < 1 ||
        cfg->batch < 64 || cfg->epochs < 0 || !(cfg->deps_sigma > 0) || !(cfg->stress_range > 0) ||
        (cfg->sampling != 0 && cfg->sampling != 1))
        return MPM_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return MPM_ERR_CUDA;
    }
    mpm_net* net = new (std::nothrow) mpm_net();
    if (!net) return MPM_ERR_NOMEM;
    net->cfg = *cfg;
    net->mat = make_mat(*cfg);
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&net->sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (cudaMalloc(&net->p, NPARAM * 4) != cudaSuccess || cudaMalloc(&net->err, 4) != cudaSuccess ||
        cudaFuncSetAttribute(k_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_TC) != cudaSuccess) {
        cudaGetLastError();
        mpm_net_destroy(net);
        return MPM_ERR_NOMEM;
    }
    cudaMemset(net->err, 0, 4);
    // initial parameters: U(-1/sqrt(fan_in), 1/sqrt(fan_in)) (padded input columns zero)
    std::vector<float> p(NPARAM, 0.0f);
    uint64_t st = cfg->seed * 0x2545F4914F6CDD1DULL + 12345;
    auto u = [&]() {
        st += 0x9e3779b97f4a7c15ULL;
        return (double)(mix64(st) >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
    };
    for (int r = 0; r < HID; ++r)
        for (int k = 0; k < NIN; ++k) p[OW1 + r * IN + k] = (float)(u() / std::sqrt((double)NIN));
    for (int r = 0; r < HID; ++r) p[OB1 + r] = (float)(u() / std::sqrt((double)NIN));
    for (long long i = 0; i < HID * HID; ++i) p[OW2 + i] = (float)(u() / std::sqrt((double)HID));
    for (int r = 0; r < HID; ++r) p[OB2 + r] = (float)(u() / std::sqrt((double)HID));
    for (long long i = 0; i < HID * HID; ++i) p[OW3 + i] = (float)(u() / std::sqrt((double)HID));
    for (int r = 0; r < HID; ++r) p[OB3 + r] = (float)(u() / std::sqrt((double)HID));
    for (long long i = 0; i < OUT * HID; ++i) p[OW4 + i] = i < NOUT * HID ? (float)(u() / std::sqrt((double)HID)) : 0.0f;
    for (int r = 0; r < NOUT; ++r) p[OB4 + r] = (float)(u() / std::sqrt((double)HID));
    if (cudaMemcpy(net->p, p.data(), NPARAM * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        mpm_net_destroy(net);
        return MPM_ERR_CUDA;
    }
    for (int c = 0; c < 6; ++c) {
        net->in_inv_scale[c] = (float)(1.0 / cfg->yield);
        net->in_inv_scale[7 + c] = (float)(1.0 / cfg->deps_sigma);
    }
    net->in_inv_scale[6] = (float)(1.0 / cfg->yield);
    for (int c = 0; c < NIN; ++c) {
        net->box_lo[c] = -INFINITY;
        net->box_hi[c] = INFINITY;
    }
    for (int c = 0; c < NOUT; ++c) {
        net->out_scale[c] = 1.0f;
        net->out_shift[c] = 0.0f;
    }
    *out = net;
    return MPM_OK;
}

void mpm_net_destroy(mpm_net* net) {
    if (!net) return;
    if (net->p) cudaFree(net->p);
    if (net->wpack) cudaFree(net->wpack);
    if (net->scratch) cudaFree(net->scratch);
    if (net->err) cudaFree(net->err);
    delete net;
}

int mpm_net_get_params(mpm_net* net, float* host, int64_t n) {
    if (!net || !host || n != NPARAM) return MPM_ERR_ARG;
    NCK(cudaMemcpy(host, net->p, NPARAM * 4, cudaMemcpyDeviceToHost));
    return MPM_OK;
}

int mpm_net_set_params(mpm_net* net, const float* host, int64_t n) {
    if (!net || !host || n != NPARAM) return MPM_ERR_ARG;
    NCK(cudaMemcpy(net->p, host, NPARAM * 4, cudaMemcpyHostToDevice));
    return pack_weights(net);
}

int mpm_net_scales(mpm_net* net, double in_scale[13], double out_scale[7], double out_shift[7]) {
    if (!net) return MPM_ERR_ARG;
    for (int c = 0; c < NIN; ++c)
        if (in_scale) in_scale[c] = 1.0 / (double)net->in_inv_scale[c];
    for (int c = 0; c < NOUT; ++c) {
        if (out_scale) out_scale[c] = net->out_scale[c];
        if (out_shift) out_shift[c] = net->out_shift[c];
    }
    return MPM_OK;
}

int mpm_net_loss_grad(mpm_net* net, const float* x, const float* t, int64_t n, float* grad, double* loss) {
    if (!net || !x || !t || !grad || n < 1) return MPM_ERR_ARG;
    const size_t fb = 4;
    const size_t need = fb * ((size_t)n * (IN + OUT + OUT + OUT) + (size_t)n * HID * 8 + NPARAM) + 64;
    int rc = ensure_scratch(net, need);
    if (rc) return rc;
    float* xs = net->scratch;
    float* ts = xs + n * IN;
    float* y = ts + n * OUT;
    float* dy = y + n * OUT;
    float* z1 = dy + n * OUT;
    float* h1 = z1 + n * HID;
    float* z2 = h1 + n * HID;
    float* h2 = z2 + n * HID;
    float* z3 = h2 + n * HID;
    float* h3 = z3 + n * HID;
    float* d1 = h3 + n * HID;
    float* d2 = d1 + n * HID;
    float* g = d2 + n * HID;
    double* dl = reinterpret_cast<double*>(((uintptr_t)(g + NPARAM) + 7) & ~(uintptr_t)7);
    cudaStream_t s = 0;
    NCK(cudaMemcpy(xs, x, (size_t)n * IN * 4, cudaMemcpyHostToDevice));
    NCK(cudaMemcpy(ts, t, (size_t)n * OUT * 4, cudaMemcpyHostToDevice));
    NCK(cudaMemset(dl, 0, 8));
    forward_fp32(net, s, n, xs, z1, h1, z2, h2, z3, h3, y);
    k_loss<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, y, ts, dy, dl);
    backward_fp32(net, s, n, xs, z1, h1, z2, h2, z3, h3, dy, d1, d2, g);
    NCK(cudaGetLastError());
    NCK(cudaMemcpy(grad, g, NPARAM * 4, cudaMemcpyDeviceToHost));
    if (loss) NCK(cudaMemcpy(loss, dl, 8, cudaMemcpyDeviceToHost));
    return MPM_OK;
}

static int train_impl(mpm_net* net, const float* d_rows, long long n_rows, mpm_net_report* rep) {
    const mpm_net_config& c = net->cfg;
    const long long nval = d_rows ? std::max(1LL, std::min(65536LL, n_rows / 20)) : std::max(65536LL, (long long)c.n_samples / 100);
    const long long n = d_rows ? n_rows - nval : (long long)c.n_samples, B = std::min<long long>(c.batch, n);
    if (n < 64) return MPM_ERR_ARG;
    mpm_net_report r;
    memset(&r, 0, sizeof(r));
    // data: x (n x 16), t (n x 8 physical), tn (n x 8 normalised), raw inputs (n x 13)
    float *x = nullptr, *t = nullptr, *tn = nullptr, *xv = nullptr, *tv = nullptr;
    auto freeall = [&]() {
        for (float* q : {x, t, tn, xv, tv})
            if (q) cudaFree(q);
    };
    if (cudaMalloc(&x, (size_t)n * IN * 4) != cudaSuccess || cudaMalloc(&t, (size_t)n * OUT * 4) != cudaSuccess ||
        cudaMalloc(&tn, (size_t)n * OUT * 4) != cudaSuccess || cudaMalloc(&xv, (size_t)nval * IN * 4) != cudaSuccess ||
        cudaMalloc(&tv, (size_t)nval * OUT * 4) != cudaSuccess) {
        cudaGetLastError();
        freeall();
        return MPM_ERR_NOMEM;
    }
    SampleCfg sc{c.yield, c.stress_range, c.epbar_max, c.deps_sigma, c.C0, c.C1, c.seed, c.sampling};
    auto t0 = std::chrono::steady_clock::now();
    if (d_rows) {
        k_label_rows<<<(unsigned)((n + 255) / 256), 256>>>(n, d_rows, sc, net->mat, x, t);
        k_label_rows<<<(unsigned)((nval + 255) / 256), 256>>>(nval, d_rows + n * NIN, sc, net->mat, xv, tv);
    } else {
        k_generate<<<(unsigned)((n + 255) / 256), 256>>>(n, 0, sc, net->mat, x, t);
        k_generate<<<(unsigned)((nval + 255) / 256), 256>>>(nval, n, sc, net->mat, xv, tv);
    }
    // output normalisation from the training set
    double* acc = nullptr;
    float* dvec = nullptr;
    if (cudaMalloc(&acc, 64 * 8) != cudaSuccess || cudaMalloc(&dvec, 64 * 4) != cudaSuccess) {
        cudaGetLastError();
        freeall();
        return MPM_ERR_NOMEM;
    }
    {  // the box of the training inputs, for the guard
        unsigned hb[2 * NIN];
        for (int c = 0; c < NIN; ++c) {
            hb[c] = 0xffffffffu;
            hb[NIN + c] = 0u;
        }
        unsigned* db = reinterpret_cast<unsigned*>(dvec);
        cudaMemcpy(db, hb, sizeof(hb), cudaMemcpyHostToDevice);
        k_box<<<net->sm_count * 4, 256>>>(n, x, db);
        cudaMemcpy(hb, db, sizeof(hb), cudaMemcpyDeviceToHost);
        for (int c = 0; c < NIN; ++c) {
            net->box_lo[c] = ord2f(hb[c]);
            net->box_hi[c] = ord2f(hb[NIN + c]);
        }
    }
    cudaMemset(acc, 0, 64 * 8);
    k_moments<<<net->sm_count * 4, 256>>>(n, t, acc);
    double h[2 * NOUT];
    cudaMemcpy(h, acc, sizeof(h), cudaMemcpyDeviceToHost);
    float fs[2 * NOUT];
    for (int k = 0; k < NOUT; ++k) {
        const double mean = h[k] / n, var = std::max(h[NOUT + k] / n - mean * mean, 1e-30);
        net->out_shift[k] = (float)mean;
        net->out_scale[k] = (float)std::sqrt(var);
        fs[k] = net->out_shift[k];
        fs[NOUT + k] = 1.0f / net->out_scale[k];
        r.out_shift[k] = net->out_shift[k];
        r.out_scale[k] = net->out_scale[k];
    }
    cudaMemcpy(dvec, fs, sizeof(fs), cudaMemcpyHostToDevice);
    k_normalise_targets<<<(unsigned)((n + 255) / 256), 256>>>(n, t, dvec, dvec + NOUT, tn);
    if (cudaDeviceSynchronize() != cudaSuccess) {
        cudaGetLastError();
        freeall();
        cudaFree(acc);
        cudaFree(dvec);
        return MPM_ERR_CUDA;
    }
    auto t1 = std::chrono::steady_clock::now();
    r.seconds_generate = std::chrono::duration<double>(t1 - t0).count();
    // training buffers
    const size_t need = 4 * ((size_t)B * (IN + 3 * OUT) + (size_t)B * HID * 8 + 3 * NPARAM) + 1024;
    int rc = ensure_scratch(net, need);
    if (rc) {
        freeall();
        cudaFree(acc);
        cudaFree(dvec);
        return rc;
    }
    float* xb = net->scratch;
    float* tb = xb + B * IN;
    float* y = tb + B * OUT;
    float* dy = y + B * OUT;
    float* z1 = dy + B * OUT;
    float* h1 = z1 + B * HID;
    float* z2 = h1 + B * HID;
    float* h2 = z2 + B * HID;
    float* z3 = h2 + B * HID;
    float* h3 = z3 + B * HID;
    float* d1 = h3 + B * HID;
    float* d2 = d1 + B * HID;
    float* g = d2 + B * HID;
    float* m1 = g + NPARAM;
    float* m2 = m1 + NPARAM;
    cudaMemset(m1, 0, 2 * NPARAM * 4);
    const long long per_epoch = n / B;
    const long long total = per_epoch * c.epochs;
    static const long long primes[] = {1000003, 2750159, 4256249, 7368787, 9999991, 15485863, 32452843,
                                       49979687, 67867967, 86028121, 104395301, 122949823};
    long long step = 0;
    cudaStream_t s = 0;
    for (int ep = 0; ep < c.epochs; ++ep) {
        long long a = primes[ep % 12];
        while (std::gcd(a, n) != 1) a += 2;
        const long long cc = (long long)(mix64(c.seed + ep) % (uint64_t)n);
        cudaMemsetAsync(acc + 32, 0, 8, s);
        for (long long b = 0; b < per_epoch; ++b, ++step) {
            k_gather<<<(unsigned)((B + 255) / 256), 256, 0, s>>>(n, x, tn, a, cc, b * B, (int)B, xb, tb);
            forward_fp32(net, s, B, xb, z1, h1, z2, h2, z3, h3, y);
            k_loss<<<(unsigned)((B + 255) / 256), 256, 0, s>>>(B, y, tb, dy, acc + 32);
            backward_fp32(net, s, B, xb, z1, h1, z2, h2, z3, h3, dy, d1, d2, g);
            // Adam, cosine-decayed step size after a short warm-up
            const double tt = (double)(step + 1);
            const double warm = std::min(1.0, tt / (double)std::max(1LL, std::min(200LL, total / 10)));
            const double lr = c.lr * warm * (0.02 + 0.98 * 0.5 * (1.0 + std::cos(3.14159265358979323846 * (double)step / (double)total)));
            const float c1 = (float)(1.0 - std::pow(0.9, tt)), c2 = (float)(1.0 - std::pow(0.999, tt));
            k_adam<<<(unsigned)((NPARAM + 255) / 256), 256, 0, s>>>(NPARAM, net->p, g, m1, m2, (float)lr, 0.9f, 0.999f,
                                                                    1e-8f, c1, c2);
        }
        double lsum = 0.0;
        cudaMemcpy(&lsum, acc + 32, 8, cudaMemcpyDeviceToHost);
        const double lmean = per_epoch ? lsum / per_epoch : 0.0;
        if (ep == 0) r.loss_first = lmean;
        r.loss_last = lmean;
    }
    if (cudaDeviceSynchronize() != cudaSuccess) {
        cudaGetLastError();
        freeall();
        cudaFree(acc);
        cudaFree(dvec);
        return MPM_ERR_CUDA;
    }
    auto t2 = std::chrono::steady_clock::now();
    r.seconds_train = std::chrono::duration<double>(t2 - t1).count();
    r.steps = step;
    // held-out errors with the FP32 forward pass
    rc = MPM_OK;
    {
        const long long chunk = std::min(nval, B);
        float fsh[2 * NOUT];
        for (int k = 0; k < NOUT; ++k) {
            fsh[k] = net->out_shift[k];
            fsh[NOUT + k] = net->out_scale[k];
        }
        cudaMemcpy(dvec, fsh, sizeof(fsh), cudaMemcpyHostToDevice);
        cudaMemset(acc, 0, 16 * 8);
        unsigned* maxbits = reinterpret_cast<unsigned*>(acc + 8);
        for (long long o = 0; o < nval; o += chunk) {
            const long long m = std::min(chunk, nval - o);
            forward_fp32(net, s, m, xv + o * IN, z1, h1, z2, h2, z3, h3, y);
            k_val_errors<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(m, y, tv + o * OUT, dvec, dvec + NOUT,
                                                                    (float)(1.0 / c.yield), 0.02f, acc, maxbits);
        }
        double v[4];
        unsigned mb = 0;
        cudaMemcpy(v, acc, sizeof(v), cudaMemcpyDeviceToHost);
        cudaMemcpy(&mb, maxbits, 4, cudaMemcpyDeviceToHost);
        float mx;
        memcpy(&mx, &mb, 4);
        r.n_val = nval;
        r.val_rms_dsig = std::sqrt(v[0] / (6.0 * nval));
        r.val_rms_dsig_outside = v[3] > 0 ? std::sqrt(v[1] / (6.0 * v[3])) : 0.0;
        r.val_max_dsig = mx;
        r.val_rms_dR = std::sqrt(v[2] / nval);
        if (cudaDeviceSynchronize() != cudaSuccess) {
            cudaGetLastError();
            rc = MPM_ERR_CUDA;
        }
    }
    freeall();
    cudaFree(acc);
    cudaFree(dvec);
    if (rc) return rc;
    rc = pack_weights(net);
    if (rep) *rep = r;
    return rc;
}

int mpm_net_train(mpm_net* net, mpm_net_report* rep) {
    if (!net) return MPM_ERR_ARG;
    return train_impl(net, nullptr, 0, rep);
}

int mpm_net_train_rows(mpm_net* net, const float* d_rows, int64_t n, mpm_net_report* rep) {
    if (!net || !d_rows || n < 128) return MPM_ERR_ARG;
    return train_impl(net, d_rows, n, rep);
}

int mpm_net_infer(mpm_net* net, const float* d_in, float* d_out, int64_t n, int kernel, void* stream) {
    if (!net || n < 0 || kernel < 0 || kernel > 3) return MPM_ERR_ARG;
    if (n == 0) return MPM_OK;
    if (!d_in || !d_out) return MPM_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    if (kernel == 2) {
        k_exact_fp32<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, d_in, net->mat, d_out);
        NCK(cudaGetLastError());
        return MPM_OK;
    }
    if (kernel == 3) {
        k_exact_wide<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, d_in, net->mat, d_out);
        NCK(cudaGetLastError());
        return MPM_OK;
    }
    if (!net->packed) {
        int rc = pack_weights(net);
        if (rc) return rc;
    }
    if (kernel == 0) {
        TcArgs a;
        a.wpack = reinterpret_cast<const uint4*>(net->wpack);
        a.bias = reinterpret_cast<const float*>((const char*)net->wpack + WBYTES);
        for (int c = 0; c < NIN; ++c) a.in_inv_scale[c] = net->in_inv_scale[c];
        for (int c = 0; c < NOUT; ++c) {
            a.out_scale[c] = net->out_scale[c];
            a.out_shift[c] = net->out_shift[c];
        }
        a.in = d_in;
        a.out = d_out;
        a.count = nullptr;
        a.n = n;
        a.err = net->err;
        a.mat = net->mat;
        const long long groups = (n + 128 * NSLOT - 1) / (128 * NSLOT);
        const unsigned grid = (unsigned)std::min<long long>(std::max<long long>(groups, 1), net->sm_count);
        k_mlp_tc<<<grid, TC_THREADS, SMEM_TC, s>>>(a);
        NCK(cudaGetLastError());
        return MPM_OK;
    }
    // FP32 reference: normalise, the training forward pass in chunks, de-normalise
    const long long chunk = std::min<long long>(n, 1 << 20);
    const size_t need = 4 * ((size_t)chunk * (IN + OUT) + (size_t)chunk * HID * 6 + 2 * NIN + 2 * NOUT) + 256;
    int rc = ensure_scratch(net, need);
    if (rc) return rc;
    float* x = net->scratch;
    float* y = x + chunk * IN;
    float* z1 = y + chunk * OUT;
    float* h1 = z1 + chunk * HID;
    float* z2 = h1 + chunk * HID;
    float* h2 = z2 + chunk * HID;
    float* z3 = h2 + chunk * HID;
    float* h3 = z3 + chunk * HID;
    float* sc = h3 + chunk * HID;
    float hs[NIN + 2 * NOUT];
    for (int c = 0; c < NIN; ++c) hs[c] = net->in_inv_scale[c];
    for (int c = 0; c < NOUT; ++c) {
        hs[NIN + c] = net->out_scale[c];
        hs[NIN + NOUT + c] = net->out_shift[c];
    }
    NCK(cudaMemcpyAsync(sc, hs, sizeof(hs), cudaMemcpyHostToDevice, s));
    for (long long o = 0; o < n; o += chunk) {
        const long long m = std::min(chunk, n - o);
        k_norm_inputs<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(m, d_in + o * NIN, sc, x);
        forward_fp32(net, s, m, x, z1, h1, z2, h2, z3, h3, y);
        k_denorm_outputs<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(m, y, sc + NIN, sc + NIN + NOUT,
                                                                     d_in + o * NIN, net->mat, d_out + o * NOUT);
    }
    NCK(cudaStreamSynchronize(s));
    return MPM_OK;
}

}  // extern "C"

namespace mpm {
int net_run_queue(mpm_net* net, const SurrogateQueue& q, cudaStream_t s, unsigned* err) {
    if (!net->packed) {
        int rc = pack_weights(net);
        if (rc) return rc;
    }
    TcArgs a;
    a.wpack = reinterpret_cast<const uint4*>(net->wpack);
    a.bias = reinterpret_cast<const float*>((const char*)net->wpack + WBYTES);
    for (int c = 0; c < NIN; ++c) a.in_inv_scale[c] = net->in_inv_scale[c];
    for (int c = 0; c < NOUT; ++c) {
        a.out_scale[c] = net->out_scale[c];
        a.out_shift[c] = net->out_shift[c];
    }
    a.in = q.in;
    a.out = q.out;
    a.count = q.count;
    a.n = q.cap;
    a.err = err;
    a.mat = net->mat;
    k_mlp_tc<<<(unsigned)net->sm_count, TC_THREADS, SMEM_TC, s>>>(a);
    return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_ERR_CUDA;
}

float net_yield(const mpm_net* net) { return (float)net->cfg.yield; }
SurrogateGuard net_guard(const mpm_net* net, float tol) {
    SurrogateGuard g;
    for (int c = 0; c < NIN; ++c) {
        g.in_inv_scale[c] = net->in_inv_scale[c];
        g.lo[c] = net->box_lo[c];
        g.hi[c] = net->box_hi[c];
    }
    g.tol = tol;
    return g;
}
const MatConst& net_material(const mpm_net* net) { return net->mat; }
}  // namespace mpm
