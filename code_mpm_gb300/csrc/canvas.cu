// GPU 2D voxel canvas (include/mpm_canvas.h): the reference's Canvas2D_CC
// voxeliser (Canvas2D_CC.cpp:5-262) as one pass over the voxels per batch of
// queued drawing operations, and an ordered compaction of the active voxels.
//
// Arithmetic follows the reference operation by operation with the _rn
// intrinsics (nothing contracted into FMAs), so voxel membership and surface
// flags are the reference's bit for bit: voxel centres ix*offset + offset/2
// (:22), distances sqrt(dx dx + dy dy) (glm::length), and for the rectangle
// and prism the local coordinates M * (x, y, 0, 1) with M = rotate(-angle, z)
// * translate(-c) formed on the host exactly as glm forms it (cos and sin of
// the host's libm; the term M[2][r] * 0 adds a signed zero and is left out).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "mpm_canvas.h"

namespace {

enum CanvasKind : int { CV_CIRCLE = 0, CV_RING, CV_RECT, CV_PRISM, CV_CUT_CIRCLE, CV_CUT_RECT };

struct CanvasOp {
    int kind;
    int pad;
    double cx, cy;  // centre (circle, ring)
    double r0, r1;  // radius (circle); r_inner + offset/2 and r_outer - offset/2 (ring)
    double ro, ri;  // ring radii
    double m00, m10, m30, m01, m11, m31;  // rows 0 and 1 of M (rectangle, prism)
    double hx, hy;                        // half sizes 0.5*sx, 0.5*sy
    double sx, half_extra;                // prism: sx and 0.5*extra
    double reach;  // circle and ring: no voxel with |dx| or |dy| above it is changed by the operation
};

constexpr int CV_THREADS = 256, CV_PER_THREAD = 16, CV_TILE = CV_THREADS * CV_PER_THREAD;

__device__ __forceinline__ double voxel_coord(unsigned i, double offset, double half) {
    return __dadd_rn(__dmul_rn((double)i, offset), half);
}

__global__ void k_canvas_apply(uint8_t* __restrict__ flags, unsigned nx, long long nvox, double offset, double half,
                               const CanvasOp* __restrict__ ops, int nops) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvox;
         v += (long long)gridDim.x * blockDim.x) {
        const double x = voxel_coord((unsigned)(v % nx), offset, half);
        const double y = voxel_coord((unsigned)(v / nx), offset, half);
        unsigned f = flags[v];
        for (int k = 0; k < nops; ++k) {
            const CanvasOp& o = ops[k];
            if (o.kind == CV_CIRCLE || o.kind == CV_CUT_CIRCLE || o.kind == CV_RING) {
                const double dx = __dadd_rn(x, -o.cx), dy = __dadd_rn(y, -o.cy);
                if (fabs(dx) > o.reach || fabs(dy) > o.reach) continue;
                const double d = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
                if (o.kind == CV_CIRCLE) {
                    if (!(d > o.r0)) f |= MPM_VOXEL_ACTIVE;
                } else if (o.kind == CV_CUT_CIRCLE) {
                    if (!(d > o.r0)) f &= ~MPM_VOXEL_ACTIVE;
                } else {
                    if (d < o.r0 || o.r1 < d) continue;
                    bool surf = fabs(__dadd_rn(d, -o.ro)) < offset || fabs(__dadd_rn(d, -o.ri)) < offset;
                    if (surf && (f & MPM_VOXEL_ACTIVE) && !(f & MPM_VOXEL_SURFACE)) surf = false;
                    f = (f | MPM_VOXEL_ACTIVE) & ~MPM_VOXEL_SURFACE;
                    if (surf) f |= MPM_VOXEL_SURFACE;
                }
            } else {
                const double lx = __dadd_rn(__dadd_rn(__dmul_rn(o.m00, x), __dmul_rn(o.m10, y)), o.m30);
                const double ly = __dadd_rn(__dadd_rn(__dmul_rn(o.m01, x), __dmul_rn(o.m11, y)), o.m31);
                if (lx < -o.hx || o.hx < lx) continue;
                if (o.kind == CV_PRISM) {
                    const double t = __dmul_rn(o.half_extra, __ddiv_rn(__dmul_rn(2.0, lx), o.sx));
                    if (ly < __dadd_rn(-o.hy, t) || __dadd_rn(o.hy, -t) < ly) continue;
                } else if (ly < -o.hy || o.hy < ly) {
                    continue;
                }
                if (o.kind == CV_CUT_RECT)
                    f &= ~MPM_VOXEL_ACTIVE;
                else
                    f |= MPM_VOXEL_ACTIVE;
            }
        }
        flags[v] = (uint8_t)f;
    }
}

// active voxels per tile of CV_TILE voxels
__global__ void __launch_bounds__(CV_THREADS) k_canvas_count(const uint8_t* __restrict__ flags, long long nvox,
                                                             unsigned* __restrict__ counts) {
    __shared__ unsigned wsum[CV_THREADS / 32];
    const long long base = blockIdx.x * (long long)CV_TILE;
    unsigned c = 0;
    for (int r = 0; r < CV_PER_THREAD; ++r) {
        const long long v = base + (long long)r * CV_THREADS + threadIdx.x;
        if (v < nvox && (flags[v] & MPM_VOXEL_ACTIVE)) ++c;
    }
    for (int off = 16; off > 0; off >>= 1) c += __shfl_down_sync(0xffffffffu, c, off);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = 0;
        for (int w = 0; w < CV_THREADS / 32; ++w) t += wsum[w];
        counts[blockIdx.x] = t;
    }
}

// write the tile's active voxels from its offset, in voxel order
__global__ void __launch_bounds__(CV_THREADS) k_canvas_write(const uint8_t* __restrict__ flags, long long nvox,
                                                             unsigned nx, double offset, double half,
                                                             const unsigned long long* __restrict__ tile_off,
                                                             double* __restrict__ xy, uint32_t* __restrict__ ids,
                                                             uint8_t* __restrict__ surface) {
    __shared__ unsigned wsum[CV_THREADS / 32];
    __shared__ unsigned long long run;
    const long long base = blockIdx.x * (long long)CV_TILE;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) run = tile_off[blockIdx.x];
    __syncthreads();
    for (int r = 0; r < CV_PER_THREAD; ++r) {
        const long long v = base + (long long)r * CV_THREADS + threadIdx.x;
        const unsigned f = v < nvox ? flags[v] : 0u;
        const bool take = (f & MPM_VOXEL_ACTIVE) != 0;
        const unsigned m = __ballot_sync(0xffffffffu, take);
        if (lane == 0) wsum[w] = __popc(m);
        __syncthreads();
        unsigned long long pos = run;
        for (int k = 0; k < w; ++k) pos += wsum[k];
        pos += __popc(m & ((1u << lane) - 1u));
        if (take) {
            if (xy) {
                xy[2 * pos] = voxel_coord((unsigned)(v % nx), offset, half);
                xy[2 * pos + 1] = voxel_coord((unsigned)(v / nx), offset, half);
            }
            if (ids) ids[pos] = (uint32_t)v;
            if (surface) surface[pos] = (uint8_t)((f & MPM_VOXEL_SURFACE) ? 1 : 0);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned t = 0;
            for (int k = 0; k < CV_THREADS / 32; ++k) t += wsum[k];
            run += t;
        }
        __syncthreads();
    }
}

}  // namespace

struct mpm_canvas {
    double width = 0, height = 0, offset = 0;
    uint32_t nx = 0, ny = 0;
    uint8_t* flags = nullptr;
    std::vector<CanvasOp> queued;
    std::string err;
};

namespace {

int canvas_fail(mpm_canvas* c, int rc, const char* fmt, ...) {
    if (c) {
        char buf[256];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        c->err = buf;
    }
    return rc;
}

#define CV_CK(call)                                                                                \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) return canvas_fail(c, MPM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

long long voxels(const mpm_canvas* c) { return (long long)c->nx * (long long)c->ny; }

// the rows 0 and 1 of rotate(-angle, z) * translate(-c), as glm forms them
void rect_transform(CanvasOp& o, double cx, double cy, double angle) {
    const double a = -angle, cs = std::cos(a), sn = std::sin(a);
    const double n[3] = {0.0, 0.0, 1.0};
    const double k[3][3] = {{0.0, -n[2], n[1]}, {n[2], 0.0, -n[0]}, {-n[1], n[0], 0.0}};
    double R[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
    for (int col = 0; col < 3; ++col)
        for (int row = 0; row < 3; ++row)
            R[col][row] = ((col == row ? cs : 0.0) + (1.0 - cs) * n[row] * n[col]) + sn * k[row][col];
    double T[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {-cx, -cy, 0.0, 1}};
    const double I[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
    double IR[4][4], M[4][4];
    auto mul = [](const double A[4][4], const double B[4][4], double C[4][4]) {
        for (int col = 0; col < 4; ++col)
            for (int row = 0; row < 4; ++row)
                C[col][row] = ((A[0][row] * B[col][0] + A[1][row] * B[col][1]) + A[2][row] * B[col][2]) +
                              A[3][row] * B[col][3];
    };
    mul(I, R, IR);
    mul(IR, T, M);
    o.m00 = M[0][0];
    o.m10 = M[1][0];
    o.m30 = M[3][0];
    o.m01 = M[0][1];
    o.m11 = M[1][1];
    o.m31 = M[3][1];
}

int queue(mpm_canvas* c, const CanvasOp& o) {
    if (!c) return MPM_ERR_ARG;
    c->queued.push_back(o);
    return MPM_OK;
}

int flush(mpm_canvas* c) {
    if (c->queued.empty()) return MPM_OK;
    CanvasOp* d_ops = nullptr;
    const size_t bytes = c->queued.size() * sizeof(CanvasOp);
    CV_CK(cudaMalloc(&d_ops, bytes));
    cudaError_t e = cudaMemcpy(d_ops, c->queued.data(), bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const long long n = voxels(c);
        const unsigned blocks = (unsigned)std::min<long long>((n + 255) / 256, 152LL * 32);
        k_canvas_apply<<<blocks, 256>>>(c->flags, c->nx, n, c->offset, 0.5 * c->offset, d_ops,
                                        (int)c->queued.size());
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
    }
    cudaFree(d_ops);
    if (e != cudaSuccess) return canvas_fail(c, MPM_ERR_CUDA, "canvas apply: %s", cudaGetErrorString(e));
    c->queued.clear();
    return MPM_OK;
}

}  // namespace

extern "C" {

int mpm_canvas_create(double width, double height, double offset, mpm_canvas** out) {
    if (!out || !(offset > 0.0) || !(width > 0.0) || !(height > 0.0)) return MPM_ERR_ARG;
    const double fx = std::floor(width / offset), fy = std::floor(height / offset);
    if (!(fx >= 1.0 && fy >= 1.0 && fx * fy < 9.0e18 && fx < 4294967295.0 && fy < 4294967295.0)) return MPM_ERR_ARG;
    mpm_canvas* c = new mpm_canvas();
    c->width = width;
    c->height = height;
    c->offset = offset;
    c->nx = (uint32_t)fx;
    c->ny = (uint32_t)fy;
    if (cudaMalloc(&c->flags, (size_t)voxels(c)) != cudaSuccess ||
        cudaMemset(c->flags, 0, (size_t)voxels(c)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(c->flags);
        delete c;
        return MPM_ERR_NOMEM;
    }
    *out = c;
    return MPM_OK;
}

int mpm_canvas_destroy(mpm_canvas* c) {
    if (!c) return MPM_ERR_ARG;
    cudaFree(c->flags);
    delete c;
    return MPM_OK;
}

int mpm_canvas_size(const mpm_canvas* c, uint32_t* nx, uint32_t* ny) {
    if (!c) return MPM_ERR_ARG;
    if (nx) *nx = c->nx;
    if (ny) *ny = c->ny;
    return MPM_OK;
}

const char* mpm_canvas_last_error(const mpm_canvas* c) { return c ? c->err.c_str() : "null canvas"; }

int mpm_canvas_draw_circle(mpm_canvas* c, double cx, double cy, double radius) {
    CanvasOp o{};
    o.kind = CV_CIRCLE;
    o.cx = cx;
    o.cy = cy;
    o.r0 = radius;
    o.reach = std::fabs(radius) * (1.0 + 1.0e-9);  // d >= |dx| up to rounding: a margin far above it
    return queue(c, o);
}

int mpm_canvas_cut_circle(mpm_canvas* c, double cx, double cy, double radius) {
    CanvasOp o{};
    o.kind = CV_CUT_CIRCLE;
    o.cx = cx;
    o.cy = cy;
    o.r0 = radius;
    o.reach = std::fabs(radius) * (1.0 + 1.0e-9);
    return queue(c, o);
}

int mpm_canvas_draw_ring(mpm_canvas* c, double cx, double cy, double radius_outer, double radius_inner) {
    if (!c) return MPM_ERR_ARG;
    CanvasOp o{};
    o.kind = CV_RING;
    o.cx = cx;
    o.cy = cy;
    o.ro = radius_outer;
    o.ri = radius_inner;
    o.r0 = radius_inner + 0.5 * c->offset;
    o.r1 = radius_outer - 0.5 * c->offset;
    o.reach = std::fabs(radius_outer);  // the ring takes d <= r_outer - offset/2
    return queue(c, o);
}

static int rect_like(mpm_canvas* c, int kind, double cx, double cy, double sx, double sy, double extra,
                     double rotation) {
    CanvasOp o{};
    o.kind = kind;
    rect_transform(o, cx, cy, rotation);
    o.hx = 0.5 * sx;
    o.hy = 0.5 * sy;
    o.sx = sx;
    o.half_extra = 0.5 * extra;
    return queue(c, o);
}

int mpm_canvas_draw_rectangle(mpm_canvas* c, double cx, double cy, double sx, double sy, double rotation) {
    return rect_like(c, CV_RECT, cx, cy, sx, sy, 0.0, rotation);
}

int mpm_canvas_draw_prism(mpm_canvas* c, double cx, double cy, double sx, double sy, double extra,
                          double rotation) {
    return rect_like(c, CV_PRISM, cx, cy, sx, sy, extra, rotation);
}

int mpm_canvas_cut_rectangle(mpm_canvas* c, double cx, double cy, double sx, double sy, double rotation) {
    return rect_like(c, CV_CUT_RECT, cx, cy, sx, sy, 0.0, rotation);
}

int mpm_canvas_flags(mpm_canvas* c, uint8_t* flags) {
    if (!c || !flags) return MPM_ERR_ARG;
    int rc = flush(c);
    if (rc) return rc;
    CV_CK(cudaMemcpy(flags, c->flags, (size_t)voxels(c), cudaMemcpyDefault));
    return MPM_OK;
}

static int tile_offsets(mpm_canvas* c, unsigned long long** d_off, unsigned long long* total) {
    const long long n = voxels(c);
    const unsigned tiles = (unsigned)((n + CV_TILE - 1) / CV_TILE);
    unsigned* d_counts = nullptr;
    CV_CK(cudaMalloc(&d_counts, (size_t)tiles * 4));
    k_canvas_count<<<tiles, CV_THREADS>>>(c->flags, n, d_counts);
    std::vector<unsigned> counts(tiles);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(counts.data(), d_counts, (size_t)tiles * 4, cudaMemcpyDeviceToHost);
    cudaFree(d_counts);
    if (e != cudaSuccess) return canvas_fail(c, MPM_ERR_CUDA, "canvas count: %s", cudaGetErrorString(e));
    std::vector<unsigned long long> off(tiles);
    unsigned long long s = 0;
    for (unsigned t = 0; t < tiles; ++t) {
        off[t] = s;
        s += counts[t];
    }
    *total = s;
    if (d_off) {
        CV_CK(cudaMalloc(d_off, (size_t)tiles * 8));
        CV_CK(cudaMemcpy(*d_off, off.data(), (size_t)tiles * 8, cudaMemcpyHostToDevice));
    }
    return MPM_OK;
}

int mpm_canvas_count_active(mpm_canvas* c, uint64_t* n) {
    if (!c || !n) return MPM_ERR_ARG;
    int rc = flush(c);
    if (rc) return rc;
    unsigned long long total = 0;
    if ((rc = tile_offsets(c, nullptr, &total))) return rc;
    *n = total;
    return MPM_OK;
}

int mpm_canvas_active_voxels(mpm_canvas* c, double* xy, uint32_t* ids, uint8_t* surface, uint64_t cap, uint64_t* n) {
    if (!c) return MPM_ERR_ARG;
    int rc = flush(c);
    if (rc) return rc;
    unsigned long long* d_off = nullptr;
    unsigned long long total = 0;
    if ((rc = tile_offsets(c, &d_off, &total))) return rc;
    if (n) *n = total;
    if (total > cap) {
        cudaFree(d_off);
        return canvas_fail(c, MPM_ERR_TOO_LARGE, "%llu active voxels, room for %llu", total,
                           (unsigned long long)cap);
    }
    // into device scratch, then to the caller's memory (host or device)
    double* d_xy = nullptr;
    uint32_t* d_ids = nullptr;
    uint8_t* d_surf = nullptr;
    cudaError_t e = cudaSuccess;
    if (total > 0) {
        if (xy && e == cudaSuccess) e = cudaMalloc(&d_xy, (size_t)total * 16);
        if (ids && e == cudaSuccess) e = cudaMalloc(&d_ids, (size_t)total * 4);
        if (surface && e == cudaSuccess) e = cudaMalloc(&d_surf, (size_t)total);
        if (e == cudaSuccess) {
            const long long nv = voxels(c);
            const unsigned tiles = (unsigned)((nv + CV_TILE - 1) / CV_TILE);
            k_canvas_write<<<tiles, CV_THREADS>>>(c->flags, nv, c->nx, c->offset, 0.5 * c->offset, d_off, d_xy,
                                                  d_ids, d_surf);
            e = cudaGetLastError();
        }
        if (xy && e == cudaSuccess) e = cudaMemcpy(xy, d_xy, (size_t)total * 16, cudaMemcpyDefault);
        if (ids && e == cudaSuccess) e = cudaMemcpy(ids, d_ids, (size_t)total * 4, cudaMemcpyDefault);
        if (surface && e == cudaSuccess) e = cudaMemcpy(surface, d_surf, (size_t)total, cudaMemcpyDefault);
    }
    cudaFree(d_xy);
    cudaFree(d_ids);
    cudaFree(d_surf);
    cudaFree(d_off);
    if (e != cudaSuccess) return canvas_fail(c, MPM_ERR_CUDA, "canvas voxels: %s", cudaGetErrorString(e));
    return MPM_OK;
}

}  // extern "C"
