// The cellular scenes' particle sets on the GPU (include/mpm_scene.h): a
// square-cell cross-section on the h/2 lattice, extruded into layers, with
// ordered compaction so the particles come out in the host generator's order
// (code_mpm_gb300/scenes.py).  Rows of the lattice (one row per x index, and
// per layer for the foam) are counted, their offsets scanned on the host
// (a few hundred thousand rows at most), and one block per row ranks its
// solid sites with warp ballots and writes their particles.  The arithmetic
// is the host generator's, operation for operation, with the _rn intrinsics:
// voxel centres (i + 1/2) s, IEEE remainder (fmod is exact) and numpy's floor
// division for positive operands.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "mpm_scene.h"

namespace {

constexpr int SG_THREADS = 256;

__device__ __forceinline__ double lattice_c(int i, double s) { return __dmul_rn(__dadd_rn((double)i, 0.5), s); }

// honeycomb: the site at lattice index i is in a wall along its axis
__device__ __forceinline__ bool hc_in(int i, double s, double pitch, double wall, double W) {
    const double c = lattice_c(i, s);
    return fmod(c, pitch) < wall && c < W;
}

__device__ __forceinline__ bool hc_solid(int ix, int iz, int n1, double s, double pitch, double wall, double W) {
    if (ix < 0 || iz < 0 || ix >= n1 || iz >= n1) return false;
    const double cx = lattice_c(ix, s), cz = lattice_c(iz, s);
    return (hc_in(ix, s, pitch, wall, W) || hc_in(iz, s, pitch, wall, W)) && cx < W && cz < W;
}

// numpy's floor division of positive doubles: div = (a - fmod(a, b)) / b,
// floor, plus one when the rounded quotient's fraction exceeds one half
__device__ __forceinline__ double floor_div_pos(double a, double b) {
    const double mod = fmod(a, b);
    const double div = __ddiv_rn(__dadd_rn(a, -mod), b);
    if (div == 0.0) return 0.0;
    double fd = floor(div);
    if (__dadd_rn(div, -fd) > 0.5) fd = __dadd_rn(fd, 1.0);
    return fd;
}

struct FoamArgs {
    double pitch, t0, t1, height, s, x0, y0, z0;
    int ncell, width, layers;
    double fx[16], fy[16];
};

// foam: the site at lattice index i is in its cell's wall along the axis with factors f, at thickness t
__device__ __forceinline__ bool fm_in(int i, double t, const double* f, const FoamArgs& a) {
    const double c = lattice_c(i, a.s);
    int k = (int)floor_div_pos(c, a.pitch);
    if (k > a.ncell) k = a.ncell;
    const double rel = __dadd_rn(c, -__dmul_rn((double)k, a.pitch));
    return rel < __dmul_rn(t, f[k]);
}

__device__ __forceinline__ double fm_thickness(int k, const FoamArgs& a) {
    const double zc = lattice_c(k, a.s);
    return __dadd_rn(a.t0, __ddiv_rn(__dmul_rn(__dadd_rn(a.t1, -a.t0), zc), a.height));
}

__device__ __forceinline__ bool fm_solid(int ix, int iy, double t, const FoamArgs& a) {
    if (ix < 0 || iy < 0 || ix >= a.width || iy >= a.width) return false;
    return fm_in(ix, t, a.fx, a) || fm_in(iy, t, a.fy, a);
}

__global__ void k_hc_count(int n1, double s, double pitch, double wall, double W, unsigned* cnt) {
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    if (ix >= n1) return;
    unsigned c = 0;
    for (int iz = 0; iz < n1; ++iz) c += hc_solid(ix, iz, n1, s, pitch, wall, W) ? 1u : 0u;
    cnt[ix] = c;
}

__global__ void k_fm_count(FoamArgs a, unsigned* cnt) {
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= (long long)a.layers * a.width) return;
    const int k = (int)(r / a.width), ix = (int)(r % a.width);
    const double t = fm_thickness(k, a);
    unsigned c = 0;
    for (int iy = 0; iy < a.width; ++iy) c += fm_solid(ix, iy, t, a) ? 1u : 0u;
    cnt[r] = c;
}

// Rank of this thread's flag among the block's set flags before it, and the block's count.
__device__ __forceinline__ unsigned block_rank(bool flag, unsigned* wsum, unsigned& total) {
    const int t = threadIdx.x, lane = t & 31, w = t >> 5, nw = blockDim.x >> 5;
    const unsigned bal = __ballot_sync(0xffffffffu, flag);
    if (lane == 0) wsum[w] = __popc(bal);
    __syncthreads();
    if (t == 0) {
        unsigned run = 0;
        for (int i = 0; i < nw; ++i) {
            const unsigned v = wsum[i];
            wsum[i] = run;
            run += v;
        }
        wsum[32] = run;
    }
    __syncthreads();
    const unsigned r = wsum[w] + __popc(bal & ((1u << lane) - 1u));
    total = wsum[32];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(SG_THREADS) k_hc_write(int n1, double s, double pitch, double wall, double W,
                                                          int layers, double ox, double oy, double oz,
                                                          const unsigned* __restrict__ off, double* __restrict__ pos,
                                                          uint8_t* __restrict__ surf, unsigned long long cap) {
    __shared__ unsigned wsum[33];
    const int ix = blockIdx.x;
    unsigned long long base = off[ix];
    const double x = __dadd_rn(ox, lattice_c(ix, s));
    for (int i0 = 0; i0 < n1; i0 += blockDim.x) {
        const int iz = i0 + threadIdx.x;
        const bool solid = iz < n1 && hc_solid(ix, iz, n1, s, pitch, wall, W);
        unsigned total;
        const unsigned r = block_rank(solid, wsum, total);
        if (solid) {
            const bool edge = !(hc_solid(ix + 1, iz, n1, s, pitch, wall, W) && hc_solid(ix - 1, iz, n1, s, pitch, wall, W) &&
                                hc_solid(ix, iz + 1, n1, s, pitch, wall, W) && hc_solid(ix, iz - 1, n1, s, pitch, wall, W));
            const double z = __dadd_rn(oz, lattice_c(iz, s));
            const unsigned long long p0 = (base + r) * (unsigned long long)layers;
            for (int j = 0; j < layers; ++j) {
                const unsigned long long p = p0 + j;
                if (p >= cap) break;
                if (pos) {
                    pos[3 * p] = x;
                    pos[3 * p + 1] = __dadd_rn(oy, lattice_c(j, s));
                    pos[3 * p + 2] = z;
                }
                if (surf) surf[p] = edge ? 1 : 0;
            }
        }
        base += total;
    }
}

__global__ void __launch_bounds__(SG_THREADS) k_fm_write(FoamArgs a, const unsigned* __restrict__ off,
                                                          double* __restrict__ pos, uint8_t* __restrict__ surf,
                                                          unsigned long long cap) {
    __shared__ unsigned wsum[33];
    const long long row = blockIdx.x;
    const int k = (int)(row / a.width), ix = (int)(row % a.width);
    const double t = fm_thickness(k, a);
    const double x = __dadd_rn(a.x0, lattice_c(ix, a.s)), z = __dadd_rn(a.z0, lattice_c(k, a.s));
    unsigned long long base = off[row];
    for (int i0 = 0; i0 < a.width; i0 += blockDim.x) {
        const int iy = i0 + threadIdx.x;
        const bool solid = iy < a.width && fm_solid(ix, iy, t, a);
        unsigned total;
        const unsigned r = block_rank(solid, wsum, total);
        if (solid) {
            const unsigned long long p = base + r;
            if (p < cap) {
                if (pos) {
                    pos[3 * p] = x;
                    pos[3 * p + 1] = __dadd_rn(a.y0, lattice_c(iy, a.s));
                    pos[3 * p + 2] = z;
                }
                if (surf) {
                    const bool edge = !(fm_solid(ix + 1, iy, t, a) && fm_solid(ix - 1, iy, t, a) &&
                                        fm_solid(ix, iy + 1, t, a) && fm_solid(ix, iy - 1, t, a));
                    surf[p] = edge ? 1 : 0;
                }
            }
        }
        base += total;
    }
}

// Scratch of one generation: row counts, and the output when the caller's buffers are host memory.
struct Scratch {
    unsigned* cnt = nullptr;
    double* pos = nullptr;
    uint8_t* surf = nullptr;
    ~Scratch() {
        cudaFree(cnt);
        cudaFree(pos);
        cudaFree(surf);
    }
};

bool is_device(const void* p) {
    if (!p) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Row counts -> exclusive row offsets (on the host) and the total.
int scan_rows(Scratch& sc, long long rows, cudaStream_t st, unsigned long long* total) {
    std::vector<unsigned> h((size_t)rows);
    if (cudaMemcpyAsync(h.data(), sc.cnt, (size_t)rows * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return MPM_ERR_CUDA;
    unsigned long long run = 0;
    for (auto& v : h) {
        const unsigned c = v;
        if (run > 0xffffffffull) return MPM_ERR_TOO_LARGE;
        v = (unsigned)run;
        run += c;
    }
    if (run > 0xffffffffull) return MPM_ERR_TOO_LARGE;
    if (cudaMemcpyAsync(sc.cnt, h.data(), (size_t)rows * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return MPM_ERR_CUDA;
    *total = run;
    return MPM_OK;
}

// Output buffers: the caller's device buffers, or scratch ones copied out afterwards.
int outputs(Scratch& sc, double* pos, uint8_t* surf, unsigned long long m, double** dpos, uint8_t** dsurf) {
    *dpos = pos;
    *dsurf = surf;
    if (pos && !is_device(pos)) {
        if (cudaMalloc(&sc.pos, (size_t)std::max(1ull, m) * 24) != cudaSuccess) return MPM_ERR_NOMEM;
        *dpos = sc.pos;
    }
    if (surf && !is_device(surf)) {
        if (cudaMalloc(&sc.surf, (size_t)std::max(1ull, m)) != cudaSuccess) return MPM_ERR_NOMEM;
        *dsurf = sc.surf;
    }
    return MPM_OK;
}

int copy_out(Scratch& sc, double* pos, uint8_t* surf, unsigned long long m, cudaStream_t st) {
    if (sc.pos && m && cudaMemcpyAsync(pos, sc.pos, (size_t)m * 24, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return MPM_ERR_CUDA;
    if (sc.surf && m && cudaMemcpyAsync(surf, sc.surf, (size_t)m, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return MPM_ERR_CUDA;
    return cudaStreamSynchronize(st) == cudaSuccess ? MPM_OK : MPM_ERR_CUDA;
}

}  // namespace

extern "C" {

int mpm_scene_honeycomb(const mpm_honeycomb_desc* d, double* pos, uint8_t* surface, uint64_t cap, uint64_t* n,
                        void* stream) {
    if (!d || !n || !(d->h > 0.0) || !(d->pitch > 0.0) || !(d->wall > 0.0) || d->ncell < 1 || d->layers < 1)
        return MPM_ERR_ARG;
    if (cudaPeekAtLastError() != cudaSuccess) return MPM_ERR_CUDA;
    const double s = 0.5 * d->h, W = d->ncell * d->pitch + d->wall;
    const double n1d = std::ceil(W / s);
    if (!(n1d >= 1.0 && n1d < 65536.0)) return MPM_ERR_ARG;
    const int n1 = (int)n1d;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (cudaMalloc(&sc.cnt, (size_t)n1 * 4) != cudaSuccess) return MPM_ERR_NOMEM;
    k_hc_count<<<(n1 + 127) / 128, 128, 0, st>>>(n1, s, d->pitch, d->wall, W, sc.cnt);
    if (cudaGetLastError() != cudaSuccess) return MPM_ERR_CUDA;
    unsigned long long sites = 0;
    int rc = scan_rows(sc, n1, st, &sites);
    if (rc) return rc;
    const unsigned long long total = sites * (unsigned long long)d->layers;
    *n = total;
    const unsigned long long m = std::min<unsigned long long>(total, cap);
    if (m == 0 || (!pos && !surface)) return MPM_OK;
    double* dpos;
    uint8_t* dsurf;
    if ((rc = outputs(sc, pos, surface, m, &dpos, &dsurf))) return rc;
    k_hc_write<<<n1, SG_THREADS, 0, st>>>(n1, s, d->pitch, d->wall, W, d->layers, d->origin[0], d->origin[1],
                                          d->origin[2], sc.cnt, dpos, dsurf, m);
    if (cudaGetLastError() != cudaSuccess) return MPM_ERR_CUDA;
    return copy_out(sc, pos, surface, m, st);
}

int mpm_scene_graded_foam(const mpm_foam_desc* d, double* pos, uint8_t* surface, uint64_t cap, uint64_t* n,
                          void* stream) {
    if (!d || !n || !d->fx || !d->fy || !(d->h > 0.0) || !(d->pitch > 0.0) || !(d->height > 0.0) || d->ncell < 1 ||
        d->ncell > 15 || d->width < 1 || d->width > 65535 || d->layers < 1)
        return MPM_ERR_ARG;
    if (cudaPeekAtLastError() != cudaSuccess) return MPM_ERR_CUDA;
    FoamArgs a;
    a.pitch = d->pitch;
    a.t0 = d->t0;
    a.t1 = d->t1;
    a.height = d->height;
    a.s = 0.5 * d->h;
    a.x0 = d->x0;
    a.y0 = d->y0;
    a.z0 = d->z0;
    a.ncell = d->ncell;
    a.width = d->width;
    a.layers = d->layers;
    for (int k = 0; k < 16; ++k) {
        a.fx[k] = k <= d->ncell ? d->fx[k] : 0.0;
        a.fy[k] = k <= d->ncell ? d->fy[k] : 0.0;
    }
    const long long rows = (long long)d->layers * d->width;
    if (rows > (1ll << 31)) return MPM_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (cudaMalloc(&sc.cnt, (size_t)rows * 4) != cudaSuccess) return MPM_ERR_NOMEM;
    k_fm_count<<<(unsigned)((rows + 127) / 128), 128, 0, st>>>(a, sc.cnt);
    if (cudaGetLastError() != cudaSuccess) return MPM_ERR_CUDA;
    unsigned long long total = 0;
    int rc = scan_rows(sc, rows, st, &total);
    if (rc) return rc;
    *n = total;
    const unsigned long long m = std::min<unsigned long long>(total, cap);
    if (m == 0 || (!pos && !surface)) return MPM_OK;
    double* dpos;
    uint8_t* dsurf;
    if ((rc = outputs(sc, pos, surface, m, &dpos, &dsurf))) return rc;
    k_fm_write<<<(unsigned)rows, SG_THREADS, 0, st>>>(a, sc.cnt, dpos, dsurf, m);
    if (cudaGetLastError() != cudaSuccess) return MPM_ERR_CUDA;
    return copy_out(sc, pos, surface, m, st);
}

}  // extern "C"
