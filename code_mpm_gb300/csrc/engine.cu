// GB300 explicit-MPM engine: context, step orchestration and the C ABI
// declared in include/mpm_gb300.h.
//
// One context owns a regular grid, its particles and every device buffer.
// All work is issued on one CUDA stream; the host only computes the
// per-step scalars (time, timeline velocity) and launches kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "kernels.cuh"
#include "run_pairs.cuh"
#include "mpm_gb300.h"
#include "mpm_surrogate.h"
#include "radix_sort.cuh"
#include "surrogate.cuh"

using namespace mpm;

namespace {

constexpr int NTHREADS = 256;

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

struct ProfRec {
    int name;
    cudaEvent_t a, b;
};

}  // namespace

struct mpm_ctx {
    int form = MPM_FORM_FP64;
    int device = 0;
    size_t tsize = 8;  // bytes of the transfer/grid real type
    Geom g{};
    double length[3]{};
    int cells[3]{};
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    // options
    int floor_friction = 0;
    int profile = 0;
    // defaults: the autotuner's choice on the 256-specimen honeycomb batch
    int p2g_reduce = 3, p2g_block = 128, pass_block = 256, gather_batch = 0;
    int pass1_corners = 2, pass1_block = 128;  // cell-run pass 1 (P2G modes 2-4)
    // simulation scalars
    mpm_sim sim{0.0, 1.0e-3, 0.0, 0.0, 10.0, 0};
    // counts
    long long n = 0;
    long long nn = 0;
    int nmat = 0;
    int ndc = 0;
    int nspec = 1;
    std::vector<Geom> geoms;
    DevBuf geom_tab, sid, alist, acount;
    bool have_alist = false;  // alist holds the active nodes of the last step
    bool grid_dirty = true;   // node values at the last step's active nodes (an output step or an upload)
    bool use_alist = false;
    std::vector<double> tl_t, tl_v;
    bool have_particles = false, have_nodes = false;
    // device buffers
    std::vector<DevBuf*> all;
    DevBuf xtab, err_word;
    // particles
    DevBuf pos, vel, fext, mass, vol, vol0, F, stress, strain, eps_p, e_strain, e_strain_max, e_strain_ti, e_plastic,
        backstress, mp_mg, strain_rate, material, pflags, dc_mult,
        Fe;  // FP64 form: elastic deformation gradient (large-strain pass 2)
    // nodes
    DevBuf g_acc, g_vel, g_ftemp, g_mg, g_state, g_fixed, g_friction, g_ratio, g_q, g_owner,
        g_nowner, g_need, g_list, g_count, rs_chunk;
    int sm_count = 152;
    DevBuf cstart, cend;
    // sort
    DevBuf keys0, vals0, keys1, vals1, keys_copy, counts;
    DevBuf dclist, mats, staging, tune_backup, surf, mon_mask, mon_acc;
    // particle-field transfers: a second staging buffer and a copy stream, so
    // one field's copy runs while the next is packed or the previous unpacked
    DevBuf staging2;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t xfer_ev[4] = {nullptr, nullptr, nullptr, nullptr};  // per buffer: copy done, kernel done
    DevBuf work_acc;  // boundary work since the last particle upload (FP64): displacement control, friction
    int nsurf = 0;
    bool have_mon = false;
    // host pinned staging for the error word
    unsigned* h_err = nullptr;
    // profiling
    std::vector<std::string> prof_names;
    std::vector<ProfRec> prof_pending;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<double> prof_ms;
    std::vector<long long> prof_cnt;
    long long launches = 0;
    const unsigned* last_perm = nullptr;
    const unsigned* last_skeys = nullptr;
    bool keys_valid = false;  // keys_copy / keys[key_buf] / loc hold the keys of the current positions
    int key_buf = 0;
    DevBuf loc;
    // return-map network (FP32 form)
    mpm_net* net = nullptr;
    float sg_band = 0.02f, sg_recheck = 0.01f;  // the network takes trial states at least sg_band k0 past the surface
    float sg_guard = 0.001f;  // tolerance of the guard on the network's results, a fraction of k0 (0: off)
    int fp64_fallback = 1;  // FP32 form: the exact map in FP64 for von Mises hardening particles near or past the surface
    unsigned sg_mats = 0;
    std::vector<MatConst> mats_host;
    DevBuf q_in, q_out, q_vol, q_pidx, q_count, sg_acc;
    // CUDA graph of two steps, replayed while nothing it captured changes
    int use_graph = 1;
    // One graph per key-buffer parity: a captured step reads the cell keys from
    // the buffer key_buf named at capture and leaves the next keys in the other,
    // so a graph is valid only while key_buf has the value it was captured with;
    // advances of odd length change the parity between replays.
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    double g_dt[2] = {0.0, 0.0};
    int g_contact[2] = {-1, -1};
    long long g_launches[2] = {0, 0};
    DevBuf dsim, tl_dev;
    double* h_sim = nullptr;  // pinned: time, dt, step (as double bits), tv[3]
    // harvesting of return-map inputs
    int hv_on = 0;
    unsigned hv_mats = 0;
    float hv_band = 0.02f;
    float* hv_rows = nullptr;
    long long hv_cap = 0;
    DevBuf hv_count;
    // particles stored in cell order (FP32 form): orig[slot] = the caller's index
    DevBuf orig, ptmp;
    bool have_orig = false, reorder_pending = false;
    int reorder_interval = 0;  // -1: never; 0: after each particle upload; N: also every N steps
    bool cell_sort = false;    // FP32 form, P2G modes 2-4: false = take the storage order as the cell order
    bool large_strain = false; // FP64 form, non-contact loop: the large-strain pass 2
    long long steps_since_reorder = 0;
    bool owner_clean = false;  // displacement-control claims all zero (phase B clears them after use)

    mpm_ctx() {
        DevBuf* list[] = {&xtab, &err_word, &pos, &vel, &fext, &mass, &vol, &vol0, &F, &stress, &strain, &eps_p,
                          &e_strain, &e_strain_max, &e_strain_ti, &e_plastic, &backstress, &mp_mg, &strain_rate,
                          &material, &pflags, &dc_mult, &g_acc, &g_vel, &g_ftemp, &g_mg,
                          &g_state, &g_fixed, &g_friction, &g_ratio, &g_q, &g_owner, &g_nowner, &g_need, &g_list, &g_count, &rs_chunk, &cstart,
                          &cend, &keys0, &vals0, &keys1, &vals1, &keys_copy, &counts, &dclist, &mats, &staging, &staging2, &tune_backup, &surf, &mon_mask, &mon_acc, &loc, &geom_tab, &sid, &alist, &acount,
                          &q_in, &q_out, &q_vol, &q_pidx, &q_count, &sg_acc, &hv_count,
                          &dsim, &tl_dev, &orig, &ptmp, &Fe, &work_acc};
        all.assign(std::begin(list), std::end(list));
    }
};

namespace {

int fail(mpm_ctx* c, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

#define CK(call)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return fail(c, MPM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

int ensure(mpm_ctx* c, DevBuf& b, size_t bytes) {
    if (b.bytes >= bytes && b.p) return MPM_OK;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(c, MPM_ERR_NOMEM, "cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
    }
    b.bytes = bytes;
    return MPM_OK;
}

template <typename T>
PView<T> pview(mpm_ctx* c) {
    PView<T> v;
    v.pos = (double*)c->pos.p;
    v.vel = (T*)c->vel.p;
    v.fext = (T*)c->fext.p;
    v.mass = (T*)c->mass.p;
    v.vol = (T*)c->vol.p;
    v.vol0 = (T*)c->vol0.p;
    v.F = (T*)c->F.p;
    v.stress = (T*)c->stress.p;
    v.strain = (T*)c->strain.p;
    v.eps_p = (T*)c->eps_p.p;
    v.e_strain = (double*)c->e_strain.p;
    v.e_strain_max = (double*)c->e_strain_max.p;
    v.e_strain_ti = (double*)c->e_strain_ti.p;
    v.e_plastic = (double*)c->e_plastic.p;
    v.backstress = (T*)c->backstress.p;
    v.mp_mg = (T*)c->mp_mg.p;
    v.strain_rate = (T*)c->strain_rate.p;
    v.material = (int32_t*)c->material.p;
    v.pflags = (uint8_t*)c->pflags.p;
    v.dc_mult = (float*)c->dc_mult.p;
    v.loc = (float*)c->loc.p;
    v.sid = c->nspec > 1 ? (const uint16_t*)c->sid.p : nullptr;
    v.orig = c->have_orig ? (const unsigned*)c->orig.p : nullptr;
    v.Fe = (double*)c->Fe.p;
    v.n = c->n;
    return v;
}

template <typename T>
NView<T> nview(mpm_ctx* c) {
    NView<T> v;
    v.acc = (T*)c->g_acc.p;
    v.vel = (T*)c->g_vel.p;
    v.ftemp = (T*)c->g_ftemp.p;
    v.mg = (T*)c->g_mg.p;
    v.state = (unsigned*)c->g_state.p;
    v.fixed = (uint8_t*)c->g_fixed.p;
    v.friction = (double*)c->g_friction.p;
    v.rec = (T*)c->g_ratio.p;
    v.q = (T*)c->g_q.p;
    v.owner = (unsigned*)c->g_owner.p;
    v.nowner = (unsigned*)c->g_nowner.p;
    v.alist = c->use_alist ? (const unsigned*)c->alist.p : nullptr;
    v.acount = (const unsigned*)c->acount.p;
    v.nn = c->nn;
    return v;
}

unsigned blocks_for(long long n, int threads = NTHREADS) {
    long long b = (n + threads - 1) / threads;
    return (unsigned)std::max<long long>(1, b);
}

// ---- profiling --------------------------------------------------------------
int prof_id(mpm_ctx* c, const char* name) {
    for (size_t i = 0; i < c->prof_names.size(); ++i)
        if (c->prof_names[i] == name) return (int)i;
    c->prof_names.push_back(name);
    c->prof_ms.push_back(0.0);
    c->prof_cnt.push_back(0);
    return (int)c->prof_names.size() - 1;
}

cudaEvent_t take_event(mpm_ctx* c) {
    if (!c->ev_pool.empty()) {
        cudaEvent_t e = c->ev_pool.back();
        c->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

struct Launch {
    mpm_ctx* c;
    int id = -1;
    cudaEvent_t a = nullptr;
    Launch(mpm_ctx* c_, const char* name) : c(c_) {
        c->launches++;
        if (c->profile) {
            id = prof_id(c, name);
            a = take_event(c);
            cudaEventRecord(a, c->stream);
        }
    }
    ~Launch() {
        if (c->profile) {
            cudaEvent_t b = take_event(c);
            cudaEventRecord(b, c->stream);
            c->prof_pending.push_back({id, a, b});
        }
    }
};

int prof_resolve(mpm_ctx* c) {
    if (c->prof_pending.empty()) return MPM_OK;
    CK(cudaStreamSynchronize(c->stream));
    for (auto& r : c->prof_pending) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, r.a, r.b);
        c->prof_ms[r.name] += ms;
        c->prof_cnt[r.name] += 1;
        c->ev_pool.push_back(r.a);
        c->ev_pool.push_back(r.b);
    }
    c->prof_pending.clear();
    return MPM_OK;
}

#define LAUNCH(name, kernel, grid, block, ...)                             \
    do {                                                                   \
        Launch l_(c, name);                                                \
        kernel<<<(grid), (block), 0, c->stream>>>(__VA_ARGS__);            \
    } while (0)
#define LAUNCH_SMEM(name, kernel, grid, block, smem, ...)                  \
    do {                                                                   \
        Launch l_(c, name);                                                \
        kernel<<<(grid), (block), (smem), c->stream>>>(__VA_ARGS__);       \
    } while (0)

// A cell-run kernel template <T, corners per thread, block size> launched for
// the runtime choice of both (1, 2 or 4 corners; 128, 256 or 512 threads).
#define LAUNCH_CELLS(name, K, T, cpt, bs, grid, smem, ...)                                              \
    do {                                                                                                \
        if ((bs) == 128) {                                                                              \
            if ((cpt) == 1) LAUNCH_SMEM(name, (K<T, 1, 128>), grid, 128, smem, __VA_ARGS__);            \
            else if ((cpt) == 2) LAUNCH_SMEM(name, (K<T, 2, 128>), grid, 128, smem, __VA_ARGS__);       \
            else LAUNCH_SMEM(name, (K<T, 4, 128>), grid, 128, smem, __VA_ARGS__);                       \
        } else if ((bs) == 256) {                                                                       \
            if ((cpt) == 1) LAUNCH_SMEM(name, (K<T, 1, 256>), grid, 256, smem, __VA_ARGS__);            \
            else if ((cpt) == 2) LAUNCH_SMEM(name, (K<T, 2, 256>), grid, 256, smem, __VA_ARGS__);       \
            else LAUNCH_SMEM(name, (K<T, 4, 256>), grid, 256, smem, __VA_ARGS__);                       \
        } else {                                                                                        \
            if ((cpt) == 1) LAUNCH_SMEM(name, (K<T, 1, 512>), grid, 512, smem, __VA_ARGS__);            \
            else if ((cpt) == 2) LAUNCH_SMEM(name, (K<T, 2, 512>), grid, 512, smem, __VA_ARGS__);       \
            else LAUNCH_SMEM(name, (K<T, 4, 512>), grid, 512, smem, __VA_ARGS__);                       \
        }                                                                                               \
    } while (0)

// ---- host-side timeline (TimeLine::getVelocity, TimeLine.h:33-46) ----------
void timeline_velocity(const mpm_ctx* c, double t, double out[3]) {
    out[0] = out[1] = out[2] = 0.0;
    int nt = (int)c->tl_t.size();
    for (int k = 0; k + 1 < nt; ++k) {
        if (c->tl_t[k] <= t && t < c->tl_t[k + 1]) {
            double s = (t - c->tl_t[k]) / (c->tl_t[k + 1] - c->tl_t[k]);
            for (int a = 0; a < 3; ++a) {
                volatile double l = (1.0 - s) * c->tl_v[3 * k + a];
                volatile double r = s * c->tl_v[3 * (k + 1) + a];
                out[a] = l + r;
            }
        }
    }
}

// ---- unpack / pack between host n x k row-major doubles and device SoA -----
// shift_identity: the FP32 form stores a 3x3 F as H = F - I (diagonal
// components 0, 4, 8 shifted by one, in FP64 before the conversion).
// Device layout: component c of item p at c * cs + p * ps (structure of arrays:
// cs = n, ps = 1; a node's interleaved accumulator record: cs = 1, ps = 8).
template <typename T>
__global__ void k_unpack(const double* __restrict__ src, T* __restrict__ dst, long long n, int k, int shift_identity,
                         long long cs, long long ps) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n * k) return;
    long long p = i / k;
    int c = (int)(i - p * k);
    double v = src[i];
    if (shift_identity && (c == 0 || c == 4 || c == 8)) v -= 1.0;
    dst[(long long)c * cs + p * ps] = (T)v;
}
// device SoA (slot order) -> host rows; with orig, slot s goes to the caller's row orig[s]
template <typename T>
__global__ void k_pack(const T* __restrict__ src, double* __restrict__ dst, long long n, int k, int shift_identity,
                       const unsigned* __restrict__ orig, long long cs, long long ps) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n * k) return;
    long long s = i / k;
    int c = (int)(i - s * k);
    double v = (double)src[(long long)c * cs + s * ps];
    if (shift_identity && (c == 0 || c == 4 || c == 8)) v += 1.0;
    dst[(orig ? (long long)orig[s] : s) * k + c] = v;
}
// dst[c n + s] = src[c n + perm[s]] for ES-byte elements (a particle field into slot order)
template <int ES>
__global__ void k_permute(const void* __restrict__ src, void* __restrict__ dst, const unsigned* __restrict__ perm,
                          long long n, int k) {
    using U = typename std::conditional<ES == 8, unsigned long long,
              typename std::conditional<ES == 4, unsigned, typename std::conditional<ES == 2, unsigned short,
                                                                                        unsigned char>::type>::type>::type;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n * k;
         i += (long long)gridDim.x * blockDim.x) {
        const long long c = i / n, s = i - c * n;
        reinterpret_cast<U*>(dst)[i] = reinterpret_cast<const U*>(src)[c * n + perm[s]];
    }
}
// dst[orig[s]] = src[s] for ES-byte single-component fields (slot order -> the caller's order)
template <int ES>
__global__ void k_scatter_orig(const void* __restrict__ src, void* __restrict__ dst, const unsigned* __restrict__ orig,
                               long long n) {
    using U = typename std::conditional<ES == 4, unsigned, unsigned char>::type;
    long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s < n) reinterpret_cast<U*>(dst)[orig[s]] = reinterpret_cast<const U*>(src)[s];
}
__global__ void k_invert(const unsigned* __restrict__ perm, unsigned* __restrict__ inv, long long n) {
    long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s < n) inv[perm[s]] = (unsigned)s;
}
__global__ void k_remap_list(unsigned* __restrict__ list, long long n, const unsigned* __restrict__ map) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) list[i] = map[list[i]];
}
__global__ void k_iota(unsigned* __restrict__ a, long long n) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) a[i] = (unsigned)i;
}
template <typename T>
__global__ void k_fill(T* __restrict__ dst, long long n, T v) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) dst[i] = v;
}
__global__ void k_identity9(void* dst, long long n, int fp64) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= 9 * n) return;
    long long c = i / n;
    double v = (c == 0 || c == 4 || c == 8) ? 1.0 : 0.0;
    if (fp64)
        ((double*)dst)[i] = v;
    else
        ((float*)dst)[i] = (float)v;
}
__global__ void k_state_u8_to_u32(const uint8_t* __restrict__ src, unsigned* __restrict__ dst, long long n) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[i];
}
__global__ void k_state_u32_to_u8(const unsigned* __restrict__ src, uint8_t* __restrict__ dst, long long n) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (uint8_t)src[i];
}
__global__ void k_mark_dc(const unsigned* __restrict__ list, int ndc, uint8_t* __restrict__ pflags) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < ndc) pflags[list[k]] |= (uint8_t)PF_IN_DC;
}
__global__ void k_compact_flag(const uint8_t* __restrict__ pflags, long long n, uint8_t bit,
                               unsigned* __restrict__ list, unsigned* __restrict__ count) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    bool take = i < n && (pflags[i] & bit);
    unsigned m = __ballot_sync(0xffffffffu, take);
    if (!m) return;
    int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(count, (unsigned)__popc(m));
    base = __shfl_sync(m, base, leader);
    if (take) list[base + __popc(m & ((1u << lane) - 1u))] = (unsigned)i;
}
// Active-node list: a block of CS_THREADS compacts a tile of CS_THREADS x
// CS_ROUNDS consecutive nodes in node order and reserves its range with one
// atomic (a counter shared by every warp would serialise tens of thousands of
// atomics at one L2 address).  Each warp takes 32 x CS_ROUNDS consecutive
// nodes, loads all its state words before counting (the loads overlap), and
// writes its entries after the warps before it.
constexpr int CS_THREADS = 256, CS_ROUNDS = 16;
__global__ void __launch_bounds__(CS_THREADS) k_compact_state(const unsigned* __restrict__ state, long long n,
                                                              unsigned bit, unsigned* __restrict__ list,
                                                              unsigned* __restrict__ count) {
    __shared__ unsigned woff[CS_THREADS / 32];
    __shared__ unsigned base;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const long long wbase = blockIdx.x * (long long)(CS_THREADS * CS_ROUNDS) + (long long)w * 32 * CS_ROUNDS;
    unsigned v[CS_ROUNDS], m[CS_ROUNDS];
#pragma unroll
    for (int r = 0; r < CS_ROUNDS; ++r) {
        const long long i = wbase + (long long)r * 32 + lane;
        v[r] = i < n ? state[i] : 0u;
    }
    unsigned cnt = 0;
#pragma unroll
    for (int r = 0; r < CS_ROUNDS; ++r) {
        m[r] = __ballot_sync(FULL_MASK, (v[r] & bit) != 0u);
        cnt += __popc(m[r]);
    }
    if (lane == 0) woff[w] = cnt;
    __syncthreads();
    if (t == 0) {
        unsigned total = 0;
        for (int k = 0; k < CS_THREADS / 32; ++k) {
            const unsigned c = woff[k];
            woff[k] = total;
            total += c;
        }
        base = total ? atomicAdd(count, total) : 0u;
    }
    __syncthreads();
    unsigned off = base + woff[w];
    const unsigned below = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < CS_ROUNDS; ++r) {
        if (v[r] & bit) list[off + __popc(m[r] & below)] = (unsigned)(wbase + (long long)r * 32 + lane);
        off += __popc(m[r]);
    }
}
// Specimen ids of an upload (int32 from the caller) to the 16-bit device
// array; the smallest index of an id outside [0, nspec) goes to *bad.
__global__ void k_specimen_ids(const int32_t* __restrict__ in, long long n, int nspec, uint16_t* __restrict__ out,
                               unsigned* __restrict__ bad) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t s = in[i];
    if (s < 0 || s >= nspec) {
        atomicMin(bad, (unsigned)i);
        return;
    }
    out[i] = (uint16_t)s;
}

__global__ void k_clear_flag(uint8_t* __restrict__ pflags, long long n, uint8_t bits) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) pflags[i] &= (uint8_t)~bits;
}

// Upload one field: host n x k doubles (or NULL -> default) into a device SoA array of the field's real type.
// Upload one field from host rows into a structure-of-arrays buffer, or with
// acc_comp >= 0 into components acc_comp .. acc_comp + k - 1 of the nodes'
// interleaved accumulator records (dst = g_acc, already allocated).
int upload_field(mpm_ctx* c, DevBuf& dst, const double* host, long long n, int k, bool fp64, double def,
                 int shift_identity = 0, int acc_comp = -1) {
    size_t esz = fp64 ? 8 : 4;
    const bool acc = acc_comp >= 0;
    const long long off = acc ? acc_comp : 0, cs = acc ? 1 : n, ps = acc ? 8 : 1;
    int rc = acc ? MPM_OK : ensure(c, dst, (size_t)n * k * esz);
    if (rc) return rc;
    if (n == 0) return MPM_OK;
    if (acc && !host) return MPM_OK;  // accumulator components are only written from host rows
    if (host) {
        rc = ensure(c, c->staging, (size_t)n * k * 8);
        if (rc) return rc;
        CK(cudaMemcpyAsync(c->staging.p, host, (size_t)n * k * 8, cudaMemcpyHostToDevice, c->stream));
        if (fp64)
            LAUNCH("unpack", k_unpack<double>, blocks_for(n * k), NTHREADS, (const double*)c->staging.p,
                   (double*)dst.p + off, n, k, shift_identity, cs, ps);
        else
            LAUNCH("unpack", k_unpack<float>, blocks_for(n * k), NTHREADS, (const double*)c->staging.p,
                   (float*)dst.p + off, n, k, shift_identity, cs, ps);
    } else if (def == 0.0) {
        CK(cudaMemsetAsync(dst.p, 0, (size_t)n * k * esz, c->stream));
    } else if (fp64) {
        LAUNCH("fill", k_fill<double>, blocks_for(n * k), NTHREADS, (double*)dst.p, n * k, def);
    } else {
        LAUNCH("fill", k_fill<float>, blocks_for(n * k), NTHREADS, (float*)dst.p, n * k, (float)def);
    }
    return MPM_OK;
}

// Download one field into host rows.  Particle fields (particles = true) go
// through the slot -> caller-index map when the slots are in cell order;
// node fields never do.
int download_field(mpm_ctx* c, const DevBuf& src, double* host, long long n, int k, bool fp64,
                   int shift_identity = 0, bool particles = false, int acc_comp = -1) {
    if (!host || n == 0) return MPM_OK;
    int rc = ensure(c, c->staging, (size_t)n * k * 8);
    if (rc) return rc;
    const unsigned* orig = (particles && c->have_orig) ? (const unsigned*)c->orig.p : nullptr;
    const bool acc = acc_comp >= 0;
    const long long off = acc ? acc_comp : 0, cs = acc ? 1 : n, ps = acc ? 8 : 1;
    if (fp64)
        LAUNCH("pack", k_pack<double>, blocks_for(n * k), NTHREADS, (const double*)src.p + off, (double*)c->staging.p,
               n, k, shift_identity, orig, cs, ps);
    else
        LAUNCH("pack", k_pack<float>, blocks_for(n * k), NTHREADS, (const float*)src.p + off, (double*)c->staging.p,
               n, k, shift_identity, orig, cs, ps);
    CK(cudaMemcpyAsync(host, c->staging.p, (size_t)n * k * 8, cudaMemcpyDeviceToHost, c->stream));
    return MPM_OK;
}

// The copy stream and events of the particle-field transfers (created once).
int xfer_ready(mpm_ctx* c) {
    if (!c->copy_stream && cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        c->copy_stream = nullptr;
        return fail(c, MPM_ERR_CUDA, "cannot create the copy stream");
    }
    for (auto& e : c->xfer_ev)
        if (!e && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            e = nullptr;
            return fail(c, MPM_ERR_CUDA, "cannot create transfer events");
        }
    return MPM_OK;
}

// Particle field i of an upload, double-buffered: the H2D copy into staging
// buffer i % 2 runs on the copy stream once that buffer's previous unpack has
// finished; the unpack on the engine stream waits for the copy.  So field
// i + 1 crosses the link while field i is unpacked.
int upload_field_pipelined(mpm_ctx* c, int i, DevBuf& dst, const double* host, long long n, int k, bool fp64,
                           double def, int shift_identity = 0) {
    if (!host || n == 0) return upload_field(c, dst, host, n, k, fp64, def, shift_identity);
    const size_t esz = fp64 ? 8 : 4, bytes = (size_t)n * k * 8;
    int rc = ensure(c, dst, (size_t)n * k * esz);
    if (rc) return rc;
    DevBuf& buf = (i & 1) ? c->staging2 : c->staging;
    if ((rc = ensure(c, buf, bytes))) return rc;
    cudaEvent_t copied = c->xfer_ev[2 * (i & 1)], unpacked = c->xfer_ev[2 * (i & 1) + 1];
    // the buffer is free once its previous unpack is done (the first two fields: once the engine stream's
    // earlier work, which may read the staging buffers, is done)
    if (i < 2) CK(cudaEventRecord(unpacked, c->stream));
    CK(cudaStreamWaitEvent(c->copy_stream, unpacked, 0));
    CK(cudaMemcpyAsync(buf.p, host, bytes, cudaMemcpyHostToDevice, c->copy_stream));
    CK(cudaEventRecord(copied, c->copy_stream));
    CK(cudaStreamWaitEvent(c->stream, copied, 0));
    if (fp64)
        LAUNCH("unpack", k_unpack<double>, blocks_for(n * k), NTHREADS, (const double*)buf.p, (double*)dst.p, n, k,
               shift_identity, n, 1);
    else
        LAUNCH("unpack", k_unpack<float>, blocks_for(n * k), NTHREADS, (const double*)buf.p, (float*)dst.p, n, k,
               shift_identity, n, 1);
    CK(cudaEventRecord(unpacked, c->stream));
    return MPM_OK;
}

// Particle field i of a download, double-buffered the other way: the pack
// into staging buffer i % 2 waits for that buffer's previous D2H copy, the
// copy on the copy stream waits for the pack.  The caller synchronises the
// copy stream once at the end.
int download_field_pipelined(mpm_ctx* c, int i, const DevBuf& src, double* host, long long n, int k, bool fp64,
                             int shift_identity) {
    if (!host || n == 0) return MPM_OK;
    DevBuf& buf = (i & 1) ? c->staging2 : c->staging;
    const size_t bytes = (size_t)n * k * 8;
    int rc = ensure(c, buf, bytes);
    if (rc) return rc;
    cudaEvent_t copied = c->xfer_ev[2 * (i & 1)], packed = c->xfer_ev[2 * (i & 1) + 1];
    if (i >= 2) CK(cudaStreamWaitEvent(c->stream, copied, 0));
    const unsigned* orig = c->have_orig ? (const unsigned*)c->orig.p : nullptr;
    if (fp64)
        LAUNCH("pack", k_pack<double>, blocks_for(n * k), NTHREADS, (const double*)src.p, (double*)buf.p, n, k,
               shift_identity, orig, n, 1);
    else
        LAUNCH("pack", k_pack<float>, blocks_for(n * k), NTHREADS, (const float*)src.p, (double*)buf.p, n, k,
               shift_identity, orig, n, 1);
    CK(cudaEventRecord(packed, c->stream));
    CK(cudaStreamWaitEvent(c->copy_stream, packed, 0));
    CK(cudaMemcpyAsync(host, buf.p, bytes, cudaMemcpyDeviceToHost, c->copy_stream));
    CK(cudaEventRecord(copied, c->copy_stream));
    return MPM_OK;
}

int check_device_error(mpm_ctx* c) {
    CK(cudaMemcpyAsync(c->h_err, c->err_word.p, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    unsigned e = *c->h_err;
    if (e) {
        CK(cudaMemsetAsync(c->err_word.p, 0, sizeof(unsigned), c->stream));
        std::string what;
        if (e & ERR_NONFINITE_POSITION) what += " non-finite particle position;";
        if (e & ERR_BAD_MATERIAL) what += " particle without a valid material;";
        if (e & ERR_WAIT_TIMEOUT) what += " a kernel's wait for its bulk copies or tensor-core work timed out;";
        return fail(c, MPM_ERR_DEVICE, "device reported:%s", what.c_str());
    }
    return MPM_OK;
}

// ---- one time step -----------------------------------------------------------
// Sort the particles by cell key: the keys of the current positions (written
// by the previous step's pass 2, or computed here after an upload), then the
// stable radix sort, whose first pass takes the identity as input values.
int sort_cells(mpm_ctx* c, const unsigned** skeys_out, const unsigned** perm_out, bool sort = true) {
    const long long n = c->n;
    const Geom& g = c->g;
    unsigned* err = (unsigned*)c->err_word.p;
    const uint16_t* sid = c->nspec > 1 ? (const uint16_t*)c->sid.p : nullptr;
    // cell keys: written by the previous step's pass 2 (which knows the new
    // positions), or computed here after an upload; then the stable radix
    // sort by key, whose first pass takes the identity as input values
    unsigned* key_src = (unsigned*)(c->key_buf ? c->keys1.p : c->keys0.p);
    unsigned* key_other = (unsigned*)(c->key_buf ? c->keys0.p : c->keys1.p);
    if (!c->keys_valid)
        LAUNCH("cell_keys", k_cell_keys, blocks_for(n), NTHREADS, (const double*)c->pos.p, n, g, key_src,
               (unsigned*)nullptr, (unsigned*)c->keys_copy.p, err,
               c->form == MPM_FORM_FP32 ? (float*)c->loc.p : (float*)nullptr, sid);
    if (!sort) {  // the slots in storage order with their keys (identity permutation)
        c->last_perm = nullptr;
        c->last_skeys = key_src;
        *skeys_out = key_src;
        *perm_out = nullptr;
        return MPM_OK;
    }
    int bits = 1;
    while (bits < 32 && ((unsigned long long)1 << bits) <= (unsigned long long)g.key_max) ++bits;
    // the fewest passes of at most 10-bit digits (27-bit keys: three 9-bit passes)
    const int passes = (bits + 9) / 10;
    const int db = std::max(8, (bits + passes - 1) / passes);
    const int nblocks = (int)((n + RS_TILE - 1) / RS_TILE);
    unsigned *kin = key_src, *vin = nullptr;
    unsigned *kout = key_other, *vout = (unsigned*)c->vals0.p;
    const int hist_total = (1 << db) * nblocks;
    const int nchunks = (hist_total + RS_SCAN_CHUNK - 1) / RS_SCAN_CHUNK;
    for (int shift = 0; shift < bits; shift += db) {
        if (db == 8)
            LAUNCH("rs_hist", k_rs_hist<8>, nblocks, RS_THREADS, kin, n, shift, (unsigned*)c->counts.p, nblocks);
        else if (db == 9)
            LAUNCH("rs_hist", k_rs_hist<9>, nblocks, RS_THREADS, kin, n, shift, (unsigned*)c->counts.p, nblocks);
        else
            LAUNCH("rs_hist", k_rs_hist<10>, nblocks, RS_THREADS, kin, n, shift, (unsigned*)c->counts.p, nblocks);
        const unsigned* chunk_prefix = nullptr;
        if (nchunks > 1) {
            LAUNCH("rs_scan", k_rs_scan_chunks, nchunks, RS_SCAN_THREADS, (unsigned*)c->counts.p, hist_total,
                   (unsigned*)c->rs_chunk.p);
            LAUNCH("rs_scan", k_rs_scan, 1, 1024, (unsigned*)c->rs_chunk.p, nchunks);
            chunk_prefix = (const unsigned*)c->rs_chunk.p;
        } else {
            LAUNCH("rs_scan", k_rs_scan, 1, 1024, (unsigned*)c->counts.p, hist_total);
        }
        if (db == 8)
            LAUNCH("rs_scatter", k_rs_scatter<8>, nblocks, RS_THREADS, kin, (const unsigned*)vin, kout, vout, n, shift,
                   (const unsigned*)c->counts.p, nblocks, chunk_prefix);
        else if (db == 9)
            LAUNCH("rs_scatter", k_rs_scatter<9>, nblocks, RS_THREADS, kin, (const unsigned*)vin, kout, vout, n, shift,
                   (const unsigned*)c->counts.p, nblocks, chunk_prefix);
        else
            LAUNCH("rs_scatter", k_rs_scatter<10>, nblocks, RS_THREADS, kin, (const unsigned*)vin, kout, vout, n,
                   shift, (const unsigned*)c->counts.p, nblocks, chunk_prefix);
        std::swap(kin, kout);
        vin = vout;
        vout = (vout == (unsigned*)c->vals0.p) ? (unsigned*)c->vals1.p : (unsigned*)c->vals0.p;
    }
    const unsigned* skeys = kin;
    const unsigned* perm = vin;
    c->last_perm = perm;
    c->last_skeys = skeys;
    *skeys_out = skeys;
    *perm_out = perm;
    return MPM_OK;
}

void graph_reset(mpm_ctx* c);

// Store the particles in cell order (FP32 form).  After a sort every
// particle array is permuted into sorted order and `orig` keeps each slot's
// index as the caller numbers it; the displacement-control list is remapped
// and the surface list rebuilt.  Later sorts find the particles nearly in
// order, so the gathers of P2G and pass 1 through the sort permutation read
// consecutive memory.  Everything the caller sees (downloads, lists, the cell
// order, last-writer claims) stays in the caller's order.
int reorder(mpm_ctx* c) {
    c->reorder_pending = false;
    c->steps_since_reorder = 0;
    const long long n = c->n;
    if (n <= 0 || c->form != MPM_FORM_FP32) return MPM_OK;
    graph_reset(c);
    const unsigned *skeys = nullptr, *perm = nullptr;
    int rc = sort_cells(c, &skeys, &perm);
    if (rc) return rc;
    if ((rc = ensure(c, c->orig, (size_t)n * 4)) || (rc = ensure(c, c->ptmp, (size_t)n * 36))) return rc;
    if (!c->have_orig) {
        LAUNCH("reorder", k_iota, blocks_for(n), NTHREADS, (unsigned*)c->orig.p, n);
        c->have_orig = true;
    }
    struct {
        DevBuf* b;
        int k, es;
    } fields[] = {{&c->pos, 3, 8},        {&c->vel, 3, 4},       {&c->fext, 3, 4},         {&c->mass, 1, 4},
                  {&c->vol, 1, 4},        {&c->vol0, 1, 4},      {&c->F, 9, 4},            {&c->stress, 6, 4},
                  {&c->strain, 6, 4},     {&c->eps_p, 6, 4},     {&c->e_strain, 1, 8},     {&c->e_strain_max, 1, 8},
                  {&c->e_strain_ti, 1, 8}, {&c->e_plastic, 1, 8}, {&c->backstress, 1, 4},   {&c->mp_mg, 3, 4},
                  {&c->strain_rate, 6, 4}, {&c->material, 1, 4}, {&c->pflags, 1, 1},       {&c->dc_mult, 1, 4},
                  {&c->loc, 3, 4},        {&c->keys_copy, 1, 4}, {&c->orig, 1, 4},         {&c->sid, 1, 2},
                  {&c->mon_mask, 1, 1}};
    const unsigned grid = (unsigned)std::min<long long>(blocks_for(n * 3), (long long)c->sm_count * 32);
    for (auto& f : fields) {
        if (f.b == &c->sid && c->nspec <= 1) continue;
        if (f.b == &c->mon_mask && !c->have_mon) continue;
        void* src = f.b->p;
        switch (f.es) {
            case 8: LAUNCH("reorder", k_permute<8>, grid, NTHREADS, src, c->ptmp.p, perm, n, f.k); break;
            case 4: LAUNCH("reorder", k_permute<4>, grid, NTHREADS, src, c->ptmp.p, perm, n, f.k); break;
            case 2: LAUNCH("reorder", k_permute<2>, grid, NTHREADS, src, c->ptmp.p, perm, n, f.k); break;
            default: LAUNCH("reorder", k_permute<1>, grid, NTHREADS, src, c->ptmp.p, perm, n, f.k); break;
        }
        CK(cudaMemcpyAsync(src, c->ptmp.p, (size_t)n * f.k * f.es, cudaMemcpyDeviceToDevice, c->stream));
    }
    // list entries: old slot -> new slot
    unsigned* inv = (unsigned*)c->ptmp.p;
    LAUNCH("reorder", k_invert, blocks_for(n), NTHREADS, perm, inv, n);
    if (c->ndc > 0) LAUNCH("reorder", k_remap_list, blocks_for(c->ndc), NTHREADS, (unsigned*)c->dclist.p, (long long)c->ndc, inv);
    CK(cudaMemsetAsync(c->g_count.p, 0, 4, c->stream));
    LAUNCH("reorder", k_compact_flag, blocks_for(n), NTHREADS, (const uint8_t*)c->pflags.p, n, (uint8_t)MPM_PF_SURFACE,
           (unsigned*)c->surf.p, (unsigned*)c->g_count.p);
    // the sorted keys are now the keys of the slots in order: they become the next sort's input
    c->key_buf = (skeys == (const unsigned*)c->keys1.p) ? 1 : 0;
    unsigned* ident = (unsigned*)(perm == (const unsigned*)c->vals0.p ? c->vals1.p : c->vals0.p);
    LAUNCH("reorder", k_iota, blocks_for(n), NTHREADS, ident, n);
    c->last_perm = ident;
    c->last_skeys = skeys;
    c->keys_valid = true;
    CK(cudaGetLastError());
    return MPM_OK;
}

// Device copy of the clock for graph replay: time, dt, step and the
// timeline velocity at the step's start, computed with the host's exact
// operations (timeline_velocity), so device and host clocks stay identical.
struct DevSim {
    double time, dt;
    unsigned long long step;
    double tv[3];
};

__global__ void k_step_begin(DevSim* d, const double* __restrict__ tl_t, const double* __restrict__ tl_v, int nt) {
    const double t = d->time;
    double out[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k + 1 < nt; ++k) {
        if (tl_t[k] <= t && t < tl_t[k + 1]) {
            const double s = __ddiv_rn(__dsub_rn(t, tl_t[k]), __dsub_rn(tl_t[k + 1], tl_t[k]));
            for (int a = 0; a < 3; ++a)
                out[a] = __dadd_rn(__dmul_rn(__dsub_rn(1.0, s), tl_v[3 * k + a]), __dmul_rn(s, tl_v[3 * (k + 1) + a]));
        }
    }
    for (int a = 0; a < 3; ++a) d->tv[a] = out[a];
}

__global__ void k_step_end(DevSim* d) {
    d->time = __dadd_rn(d->time, d->dt);
    d->step += 1;
}

void graph_reset(mpm_ctx* c) {
    for (int k = 0; c && k < 2; ++k) {
        if (!c->gexec[k]) continue;
        cudaGraphExecDestroy(c->gexec[k]);
        c->gexec[k] = nullptr;
    }
}

// output: the step is an output step, the last of an advance, whose results
// the caller can see.  Only an output step runs the contact path's contact
// detection (node mass gradients, particle and node normals, node contact
// flags, …_Contact.cpp:126-237) and writes the contact path's strain rate
// (:509): both are output only, as nothing in a step reads them
// (GridPoint.h:17-18 marks the flags as graphics debugging) and each step
// recomputes them from that step's particles.  Only an output step keeps its
// node values: the others zero their active nodes once the records are formed
// (pass 2 reads only the records), so the next step needs no grid reset.
template <typename T>
int step_impl(mpm_ctx* c, double dt, int contact, bool graph, bool output) {
    const long long n = c->n, nn = c->nn;
    PView<T> P = pview<T>(c);
    NView<T> N = nview<T>(c);
    const Geom& g = c->g;
    unsigned* err = (unsigned*)c->err_word.p;

    DevSim* dsim = (DevSim*)c->dsim.p;
    if (graph) LAUNCH("step_clock", k_step_begin, 1, 1, dsim, (const double*)c->tl_dev.p, (const double*)c->tl_dev.p + c->tl_t.size(), (int)c->tl_t.size());
    // node kernels sweep the active-node list; the reset uses the previous step's
    const unsigned nodeblocks = (unsigned)std::min<long long>(blocks_for(nn), (long long)c->sm_count * 16);
    N.alist = c->have_alist ? (const unsigned*)c->alist.p : nullptr;
    // after an upload the reset clears the uploaded active nodes only
    const int vel_zero = c->have_alist ? 1 : 0;
    if (c->grid_dirty) {  // after a step that left its node values (or an upload); clean steps zero their own
        LAUNCH("reset_grid", k_reset_grid<T>, c->have_alist ? nodeblocks : blocks_for(nn), NTHREADS, N, contact);
        c->grid_dirty = false;
    }
    if (n > 0) {
        // The FP32 form's cell-run kernels accept slots out of cell order (a
        // cell met twice is summed in two runs), so with particles stored in
        // cell order it can skip the sort and take the storage order as it is.
        const bool sort = !(c->form == MPM_FORM_FP32 && !c->cell_sort && c->p2g_reduce >= 2);
        const unsigned *skeys = nullptr, *perm = nullptr;
        if (int rs = sort_cells(c, &skeys, &perm, sort)) return rs;
        // pass 2 writes the next step's sort input into the buffer not holding skeys
        unsigned* keys_next = (skeys == (unsigned*)c->keys0.p) ? (unsigned*)c->keys1.p : (unsigned*)c->keys0.p;
        c->key_buf = (keys_next == (unsigned*)c->keys1.p) ? 1 : 0;
        const unsigned* keys = (const unsigned*)c->keys_copy.p;
        // FP32 form: the contact mass gradient is accumulated by P2G itself
        // and P2G marks the active nodes; the FP64 form marks them here and
        // records the per-cell ranges its bit-exact ordered gather reads.
        const int fp32 = c->form == MPM_FORM_FP32 ? 1 : 0;
        const bool detecting = contact && output;
        const int mg_in_p2g = (detecting && fp32) ? 1 : 0;
        if (!fp32) {
            if (detecting) {
                CK(cudaMemsetAsync(c->cstart.p, 0, (size_t)g.key_max * 4, c->stream));
                CK(cudaMemsetAsync(c->cend.p, 0, (size_t)g.key_max * 4, c->stream));
            }
            LAUNCH("cell_ranges", k_cell_ranges, blocks_for(n), NTHREADS, skeys, n, g, N.state,
                   detecting ? (unsigned*)c->cstart.p : nullptr, detecting ? (unsigned*)c->cend.p : nullptr, perm,
                   P.sid);
        }
        bool pairs_done = false;
        if constexpr (sizeof(T) == 4) {
            if (c->p2g_reduce >= 5) {  // runs reduced in registers and by a pair shuffle (mode 6: tile staged)
                const int bs = c->p2g_block;
                const unsigned pg = (unsigned)((n + 4LL * bs - 1) / (4LL * bs));
                const bool st = c->p2g_reduce == 6;
#define PAIRS(B, MGV, STV)                                                                                       \
    LAUNCH_SMEM("p2g", (k_p2g_pairs<B, MGV, STV>), pg, B, p2g_pairs_smem<B>(STV), P, N, g, skeys, perm, n, 1, err)
#define PAIRS_BS(B)                            \
    do {                                       \
        if (mg_in_p2g) {                       \
            if (st) PAIRS(B, true, true);      \
            else PAIRS(B, true, false);        \
        } else {                               \
            if (st) PAIRS(B, false, true);     \
            else PAIRS(B, false, false);       \
        }                                      \
    } while (0)
                if (bs == 128) PAIRS_BS(128);
                else if (bs == 256) PAIRS_BS(256);
                else PAIRS_BS(512);
#undef PAIRS_BS
#undef PAIRS
                pairs_done = true;
            }
        }
        if (pairs_done) {
        } else if (c->p2g_reduce >= 2) {  // shared-memory cell runs, 1 / 2 / 4 corners per thread
            const int bs = c->p2g_block, cpt = 1 << std::min(2, c->p2g_reduce - 2);
            if (mg_in_p2g)
                LAUNCH_CELLS("p2g", k_p2g_cells_mg, T, cpt, bs, blocks_for(n, bs), p2g_cells_smem<T>(bs), P, N, g,
                             skeys, perm, n, fp32);
            else
                LAUNCH_CELLS("p2g", k_p2g_cells, T, cpt, bs, blocks_for(n, bs), p2g_cells_smem<T>(bs), P, N, g, skeys,
                             perm, n, fp32);
        }
        else if (c->p2g_reduce == 1)
            LAUNCH("p2g", (k_p2g<T, 1>), blocks_for(n, c->p2g_block), c->p2g_block, P, N, g, skeys, perm, n,
                   mg_in_p2g, fp32);
        else
            LAUNCH("p2g", (k_p2g<T, 0>), blocks_for(n, c->p2g_block), c->p2g_block, P, N, g, skeys, perm, n,
                   mg_in_p2g, fp32);
        CK(cudaMemsetAsync(c->acount.p, 0, 4, c->stream));
        LAUNCH("active_list", k_compact_state, (unsigned)((nn + CS_THREADS * CS_ROUNDS - 1) / (CS_THREADS * CS_ROUNDS)),
               CS_THREADS, (const unsigned*)N.state, nn, 1u, (unsigned*)c->alist.p, (unsigned*)c->acount.p);
        N.alist = (const unsigned*)c->alist.p;
        c->have_alist = true;
        if (c->ndc > 0) {
            if (!c->owner_clean) CK(cudaMemsetAsync(c->g_owner.p, 0, (size_t)3 * nn * 4, c->stream));
            c->owner_clean = false;  // claims in use until phase B clears them
            LAUNCH("dc_claim", k_dc_claim, blocks_for(c->ndc), NTHREADS, (const unsigned*)c->dclist.p, c->ndc, keys,
                   (const uint8_t*)c->pflags.p, g, (unsigned*)c->g_owner.p, nn, contact, P.sid, (unsigned*)N.state);
        }
        if (detecting) {
            const unsigned* surf = (const unsigned*)c->surf.p;
            const int ns = c->nsurf;
            const unsigned sb = blocks_for(ns);
            if (!mg_in_p2g) {
                CK(cudaMemsetAsync(c->g_need.p, 0, (size_t)nn * 4, c->stream));
                CK(cudaMemsetAsync(c->g_count.p, 0, 4, c->stream));
                if (ns > 0)
                    LAUNCH("contact_need", k_contact_need<T>, sb, NTHREADS, P, keys, g, (unsigned*)c->g_need.p, surf,
                           ns);
                LAUNCH("contact_compact", k_contact_compact, blocks_for(nn), NTHREADS, (const unsigned*)c->g_need.p,
                       nn, (unsigned*)c->g_list.p, (unsigned*)c->g_count.p);
                LAUNCH("contact_mass_gradient", k_contact_mass_gradient<T>, (unsigned)c->sm_count * 8, CG_WARPS * 32,
                       P, N, g, (const unsigned*)c->g_list.p, (const unsigned*)c->g_count.p, perm,
                       (const unsigned*)c->cstart.p, (const unsigned*)c->cend.p);
            }
            if (ns > 0)
                LAUNCH("contact_mp_gradient", k_contact_mp_gradient<T>, sb, NTHREADS, P, N, g, keys, surf, ns);
            LAUNCH("contact_reset", k_contact_reset<T>, nodeblocks, NTHREADS, N);
            if (ns > 0) {
                LAUNCH("contact_normal", k_contact_normal<T>, sb, NTHREADS, P, N, g, keys, surf, ns, 0);
                LAUNCH("contact_normal", k_contact_normal<T>, sb, NTHREADS, P, N, g, keys, surf, ns, 1);
                LAUNCH("contact_flags", k_contact_flags<T>, sb, NTHREADS, P, N, g, keys, surf, ns);
            }
        }
        // the mass threshold in the form's type (FP32: rounded down, so float masses compare exactly)
        const T mm = sizeof(T) == 4 ? (T)fps_float_threshold(c->sim.mass_min) : (T)c->sim.mass_min;
        // displacement control, grid update, displacement control, f/m: one pass over the active nodes
        LAUNCH("node_phase_a", k_node_phase_a<T>, nodeblocks, NTHREADS, N, (T)dt, c->sim.damping, contact,
               c->floor_friction, (const unsigned*)c->dclist.p, c->ndc, (const T*)c->vel.p, n, mm, output ? 0 : 1,
               (double*)c->work_acc.p, dt);
        if (sizeof(T) == 4 && c->p2g_reduce >= 5) {  // the same runs as P2G, reduced by lane pairs
            if constexpr (sizeof(T) == 4) {
                const int b1 = c->pass1_block;
                const unsigned pg = (unsigned)((n + 4LL * b1 - 1) / (4LL * b1));
                if (b1 == 128)
                    LAUNCH("pass1_remap", k_pass1_pairs<128>, pg, 128, P, N, g, skeys, perm, n, (float)dt, contact);
                else if (b1 == 256)
                    LAUNCH("pass1_remap", k_pass1_pairs<256>, pg, 256, P, N, g, skeys, perm, n, (float)dt, contact);
                else
                    LAUNCH("pass1_remap", k_pass1_pairs<512>, pg, 512, P, N, g, skeys, perm, n, (float)dt, contact);
            }
        } else if (c->p2g_reduce >= 2) {  // the same reduction as P2G: shared-memory cell runs
            const int b1 = c->pass1_block;
            LAUNCH_CELLS("pass1_remap", k_pass1_cells, T, c->pass1_corners, b1, blocks_for(n, b1),
                         pass1_cells_smem<T>(b1), P, N, g, skeys, perm, n, (T)dt, mm, contact);
        }
        else if (c->gather_batch)
            LAUNCH("pass1_remap", (k_pass1_remap<T, 1>), blocks_for(n), NTHREADS, P, N, g, skeys, perm, n, (T)dt, mm,
                   contact);
        else
            LAUNCH("pass1_remap", (k_pass1_remap<T, 0>), blocks_for(n), NTHREADS, P, N, g, skeys, perm, n, (T)dt, mm,
                   contact);
        // remap, displacement control and BC in the path's order, p/m and v: one pass
        LAUNCH("node_phase_b", k_node_phase_b<T>, nodeblocks, NTHREADS, N, contact, (const unsigned*)c->dclist.p,
               c->ndc, (const T*)c->vel.p, n, mm, output ? 0 : 1, vel_zero);
        if (output) c->grid_dirty = true;  // the last step of an advance keeps its node values for the caller
        if (c->ndc > 0) c->owner_clean = true;
        StepArgs a;
        a.dt = dt;
        a.mass_min = c->sim.mass_min;
        a.dt_f = (float)dt;
        a.mass_min_f = fps_float_threshold(c->sim.mass_min);
        timeline_velocity(c, c->sim.time, a.tv);
        a.tv_dev = graph ? dsim->tv : nullptr;
        a.has_timeline = c->tl_t.empty() ? 0 : 1;
        a.contact = contact;
        a.sg_on = 0;
        a.sg_mats = 0;
        a.sg_band = 0.0f;
        a.q = SurrogateQueue{};
        a.sg_acc = nullptr;
        a.fb_wide = (sizeof(T) == 4 && c->fp64_fallback) ? 1 : 0;
        a.fb_below = 1.0e-3f;  // FP32 rounding of the trial yield function is below 1e-5 k0
        a.hv_on = c->hv_on;
        a.hv_mats = c->hv_mats;
        a.hv_band = c->hv_band;
        a.hv_rows = c->hv_rows;
        a.hv_count = (unsigned*)c->hv_count.p;
        a.hv_cap = c->hv_cap;
        a.outputs = output ? 1 : 0;
        const bool use_net = sizeof(T) == 4 && c->net && c->sg_mats;
        if (use_net) {
            int rq;
            if ((rq = ensure(c, c->q_in, (size_t)n * 13 * 4)) || (rq = ensure(c, c->q_out, (size_t)n * 7 * 4)) ||
                (rq = ensure(c, c->q_vol, (size_t)n * 4)) || (rq = ensure(c, c->q_pidx, (size_t)n * 4)) ||
                (rq = ensure(c, c->q_count, 64)))
                return rq;
            CK(cudaMemsetAsync(c->q_count.p, 0, 4, c->stream));
            a.sg_on = 1;
            a.sg_mats = c->sg_mats;
            a.sg_band = c->sg_band;
            a.q = SurrogateQueue{(float*)c->q_in.p, (float*)c->q_out.p, (float*)c->q_vol.p, (unsigned*)c->q_pidx.p,
                                 (unsigned*)c->q_count.p, n};
            a.sg_acc = (SurrogateAcc*)c->sg_acc.p;
        }
        {
            const unsigned pb = blocks_for(n, c->pass_block);
            unsigned* kc = (unsigned*)c->keys_copy.p;
            const MatConst* mats = (const MatConst*)c->mats.p;
#define PASS2(B, S) LAUNCH("pass2", (k_pass2<T, B, S>), pb, S, P, N, g, kc, keys_next, mats, c->nmat, a, err)
            bool large = false;
            if constexpr (sizeof(T) == 8) {
                if (c->large_strain && !contact) {  // non-contact loop only, as in the reference
                    LAUNCH("pass2", k_pass2_ls<128>, blocks_for(n, 128), 128, P, N, g, kc, keys_next, mats, c->nmat,
                           a, err);
                    large = true;
                }
            }
            if (large) {
            } else if (c->gather_batch == 2 && sizeof(T) == 4) {
                if constexpr (sizeof(T) == 4) {
                    if (c->pass_block == 128)
                        LAUNCH_SMEM("pass2", k_pass2_staged<128>, pb, 128, Pass2Stage<128>::SMEM, P, N, g, kc,
                                    keys_next, mats, c->nmat, a, err);
                    else if (c->pass_block == 256)
                        LAUNCH_SMEM("pass2", k_pass2_staged<256>, pb, 256, Pass2Stage<256>::SMEM, P, N, g, kc,
                                    keys_next, mats, c->nmat, a, err);
                    else
                        LAUNCH_SMEM("pass2", k_pass2_staged<512>, pb, 512, Pass2Stage<512>::SMEM, P, N, g, kc,
                                    keys_next, mats, c->nmat, a, err);
                }
            } else if (c->pass_block == 128) {
                if (c->gather_batch == 1) PASS2(1, 128); else PASS2(0, 128);
            } else if (c->pass_block == 256) {
                if (c->gather_batch == 1) PASS2(1, 256); else PASS2(0, 256);
            } else {
                if (c->gather_batch == 1) PASS2(1, 512); else PASS2(0, 512);
            }
#undef PASS2
        }
        if constexpr (sizeof(T) == 4) {
            if (use_net) {
                int rq;
                {
                    Launch l_(c, "net_infer");
                    rq = net_run_queue(c->net, a.q, c->stream, err);
                }
                if (rq) return rq;
                LAUNCH("net_finish", k_sg_finish, (unsigned)c->sm_count * 8, 256, P, a.q, net_material(c->net),
                       contact, dt, 1.0 / (double)net_yield(c->net), c->sg_recheck, (unsigned long long)c->sim.step,
                       graph ? &dsim->step : (const unsigned long long*)nullptr, a.sg_acc,
                       net_guard(c->net, c->sg_guard));
            }
        }
        c->keys_valid = true;
    }
    if (graph) LAUNCH("step_clock", k_step_end, 1, 1, dsim);
    c->steps_since_reorder += 1;
    CK(cudaGetLastError());
    // d_Time += dTimeIncrement; i_TimeCycle++ (…MPLocks.cpp:802-803)
    c->sim.time += dt;
    c->sim.step += 1;
    return MPM_OK;
}

int step(mpm_ctx* c, double dt, int contact, bool graph = false, bool output = true) {
    return c->form == MPM_FORM_FP64 ? step_impl<double>(c, dt, contact, graph, output)
                                    : step_impl<float>(c, dt, contact, graph, output);
}

// Steps nsteps with the two-step graph where it applies: the steady state
// (keys from the previous pass 2, an active-node list), no profiling, a
// stream that can be captured, the same dt and contact flag as the cached
// graph.  Capturing records two steps without running them while the host
// state advances by two steps; launching the graph once then brings the
// device to the same point.
// Steps between periodic reorders (FP32 form; 0: none).  Without the
// per-step sort the storage order is the only cell order, so it is restored
// every SORT_FREE_REORDER steps unless the caller chose an interval.
constexpr int SORT_FREE_REORDER = 256;
int reorder_every(const mpm_ctx* c) {
    if (c->form != MPM_FORM_FP32 || c->reorder_interval < 0) return 0;
    if (c->reorder_interval > 0) return c->reorder_interval;
    return (!c->cell_sort && c->p2g_reduce >= 2) ? SORT_FREE_REORDER : 0;
}

int advance_graph(mpm_ctx* c, int nsteps, double dt, int contact, bool between_reorders = false,
                  bool output_last = true) {
    if (!between_reorders) {
        if (c->reorder_pending && c->have_particles) {
            int rc = reorder(c);
            if (rc) return rc;
        }
        const int every = reorder_every(c);
        if (every > 0) {  // periodic: advance in runs between reorders
            while (nsteps > 0) {
                const long long left = std::max<long long>(1, every - c->steps_since_reorder);
                const int k = (int)std::min<long long>(nsteps, left);
                int rc = advance_graph(c, k, dt, contact, true, output_last && k == nsteps);
                if (rc) return rc;
                nsteps -= k;
                if (c->steps_since_reorder >= every && (rc = reorder(c))) return rc;
            }
            return MPM_OK;
        }
    }
    int s = 0;
    auto one = [&]() -> int { return step(c, dt, contact, false, output_last && s == nsteps - 1); };
    // launches the remaining steps one by one, the last as the output step
    auto plain = [&]() -> int {
        for (; s < nsteps; ++s)
            if (int rc = one()) return rc;
        return MPM_OK;
    };
    while (s < nsteps && (!c->keys_valid || !c->have_alist || c->grid_dirty)) {
        if (int rc = one()) return rc;
        ++s;
    }
    // the graph's steps are not output steps (no contact detection, node values zeroed after use); the last
    // step then runs plainly as the output step
    const int tail = output_last ? 1 : 0;
    const bool can = c->use_graph && !c->profile && c->stream != nullptr && c->n > 0 && nsteps - tail - s >= 2;
    if (!can) return plain();
    const int par = c->key_buf;  // the capture's two steps flip it twice: the same on return
    if (c->gexec[par] && (c->g_dt[par] != dt || c->g_contact[par] != contact)) graph_reset(c);
    int rc;
    if ((rc = ensure(c, c->dsim, sizeof(DevSim)))) return rc;
    if (!c->h_sim && cudaMallocHost(&c->h_sim, sizeof(DevSim)) != cudaSuccess) {
        cudaGetLastError();
        return plain();
    }
    // the device clock from the host's
    CK(cudaStreamSynchronize(c->stream));
    DevSim hs{c->sim.time, dt, (unsigned long long)c->sim.step, {0.0, 0.0, 0.0}};
    memcpy(c->h_sim, &hs, sizeof(hs));
    CK(cudaMemcpyAsync(c->dsim.p, c->h_sim, sizeof(DevSim), cudaMemcpyHostToDevice, c->stream));
    if (!c->gexec[par]) {
        const long long l0 = c->launches;
        cudaGraph_t gr = nullptr;
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
        int r1 = step(c, dt, contact, true, false);
        int r2 = r1 ? r1 : step(c, dt, contact, true, false);
        cudaError_t ec = cudaStreamEndCapture(c->stream, &gr);
        if (r2 || ec != cudaSuccess) {
            cudaGetLastError();
            if (gr) cudaGraphDestroy(gr);
            return r2 ? r2 : fail(c, MPM_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(ec));
        }
        ec = cudaGraphInstantiate(&c->gexec[par], gr, 0);
        cudaGraphDestroy(gr);
        if (ec != cudaSuccess) {
            cudaGetLastError();
            c->gexec[par] = nullptr;
            return fail(c, MPM_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(ec));
        }
        if (c->key_buf != par) return fail(c, MPM_ERR_STATE, "captured steps left the key buffers out of phase");
        c->g_dt[par] = dt;
        c->g_contact[par] = contact;
        c->g_launches[par] = c->launches - l0;
        CK(cudaGraphLaunch(c->gexec[par], c->stream));  // the two captured steps (host state already advanced)
        s += 2;
    }
    for (; nsteps - tail - s >= 2; s += 2) {
        CK(cudaGraphLaunch(c->gexec[par], c->stream));
        c->launches += c->g_launches[par];
        c->steps_since_reorder += 2;
        c->sim.time += dt;
        c->sim.step += 1;
        c->sim.time += dt;
        c->sim.step += 1;
    }
    return plain();
}

int alloc_particles(mpm_ctx* c, long long n) {
    const size_t t = c->tsize;
    struct {
        DevBuf* b;
        size_t bytes;
    } plan[] = {{&c->pos, 3 * 8},     {&c->vel, 3 * t},        {&c->fext, 3 * t},        {&c->mass, t},
                {&c->vol, t},         {&c->vol0, t},           {&c->F, 9 * t},           {&c->stress, 6 * t},
                {&c->strain, 6 * t},  {&c->eps_p, 6 * t},      {&c->e_strain, 8},        {&c->e_strain_max, 8},
                {&c->e_strain_ti, 8}, {&c->e_plastic, 8},      {&c->backstress, t},      {&c->mp_mg, 3 * t},
                {&c->strain_rate, 6 * t}, {&c->material, 4},   {&c->pflags, 1},          {&c->dc_mult, 4},
                {&c->Fe, c->form == MPM_FORM_FP64 ? 72u : 0u},
                {&c->keys0, 4},       {&c->vals0, 4},          {&c->keys1, 4},           {&c->vals1, 4},
                {&c->keys_copy, 4},   {&c->loc, c->form == MPM_FORM_FP32 ? 12u : 0u}};
    for (auto& e : plan) {
        int rc = ensure(c, *e.b, (size_t)n * e.bytes);
        if (rc) return rc;
    }
    const long long nblocks = std::max<long long>(1, (n + RS_TILE - 1) / RS_TILE);
    int rc = ensure(c, c->counts, (size_t)1024 * nblocks * 4);
    if (rc) return rc;
    const long long nchunks = (1024 * nblocks + RS_SCAN_CHUNK - 1) / RS_SCAN_CHUNK;
    return ensure(c, c->rs_chunk, (size_t)std::max<long long>(1, nchunks) * 4);
}

}  // namespace

// =============================================================================
// C ABI
// =============================================================================
// The cell-run kernels stage up to 512 slots in shared memory (P2G: 123 KB
// in FP64, pass 1: 54 KB): allow each instantiation its dynamic shared memory.
template <typename T, int CPT, int BS>
bool cells_attr() {
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    return cudaFuncSetAttribute(k_p2g_cells<T, CPT, BS>, a, (int)p2g_cells_smem<T>(BS)) == cudaSuccess &&
           cudaFuncSetAttribute(k_p2g_cells_mg<T, CPT, BS>, a, (int)p2g_cells_smem<T>(BS)) == cudaSuccess &&
           cudaFuncSetAttribute(k_pass1_cells<T, CPT, BS>, a, (int)pass1_cells_smem<T>(BS)) == cudaSuccess;
}
template <int BS>
bool pairs_attr() {
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    return cudaFuncSetAttribute(k_p2g_pairs<BS, false, false>, a, (int)p2g_pairs_smem<BS>(false)) == cudaSuccess &&
           cudaFuncSetAttribute(k_p2g_pairs<BS, true, false>, a, (int)p2g_pairs_smem<BS>(false)) == cudaSuccess &&
           cudaFuncSetAttribute(k_p2g_pairs<BS, false, true>, a, (int)p2g_pairs_smem<BS>(true)) == cudaSuccess &&
           cudaFuncSetAttribute(k_p2g_pairs<BS, true, true>, a, (int)p2g_pairs_smem<BS>(true)) == cudaSuccess;
}
bool pass2_staged_attrs() {
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    return cudaFuncSetAttribute(k_pass2_staged<128>, a, Pass2Stage<128>::SMEM) == cudaSuccess &&
           cudaFuncSetAttribute(k_pass2_staged<256>, a, Pass2Stage<256>::SMEM) == cudaSuccess &&
           cudaFuncSetAttribute(k_pass2_staged<512>, a, Pass2Stage<512>::SMEM) == cudaSuccess;
}
template <typename T>
bool cells_attrs() {
    return cells_attr<T, 1, 128>() && cells_attr<T, 2, 128>() && cells_attr<T, 4, 128>() &&
           cells_attr<T, 1, 256>() && cells_attr<T, 2, 256>() && cells_attr<T, 4, 256>() &&
           cells_attr<T, 1, 512>() && cells_attr<T, 2, 512>() && cells_attr<T, 4, 512>();
}

extern "C" {

int mpm_device_info(char* name, int name_len, int* sm_count, int* cc_major, int* cc_minor) {
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return MPM_ERR_CUDA;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return MPM_ERR_CUDA;
    if (name && name_len > 0) {
        strncpy(name, prop.name, (size_t)name_len - 1);
        name[name_len - 1] = 0;
    }
    if (sm_count) *sm_count = prop.multiProcessorCount;
    if (cc_major) *cc_major = prop.major;
    if (cc_minor) *cc_minor = prop.minor;
    return MPM_OK;
}

int mpm_create(const mpm_grid_desc* grid, int form, mpm_ctx** out) { return mpm_create_batch(grid, 1, form, out); }

int mpm_create_batch(const mpm_grid_desc* grids, int32_t nspec, int form, mpm_ctx** out) {
    if (!out) return MPM_ERR_ARG;
    *out = nullptr;
    if (!grids || nspec < 1 || nspec > 65535 || (form != MPM_FORM_FP64 && form != MPM_FORM_FP32)) return MPM_ERR_ARG;
    long long keyspace = 0, nodes = 0;
    for (int s = 0; s < nspec; ++s) {
        long long ks = 1, ns = 1;
        for (int a = 0; a < 3; ++a) {
            const mpm_grid_desc& gd = grids[s];
            if (!(gd.length[a] > 0.0) || !std::isfinite(gd.length[a]) || gd.cells[a] < 1) return MPM_ERR_ARG;
            ks *= (long long)gd.cells[a] + 2;
            ns *= (long long)gd.cells[a] + 1;
        }
        keyspace += ks;
        nodes += ns;
    }
    if (keyspace >= 0xffffffffLL || nodes >= 0xffffffffLL) return MPM_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return MPM_ERR_CUDA;
    }
    mpm_ctx* c = new mpm_ctx();
    c->form = form;
    c->tsize = form == MPM_FORM_FP64 ? 8 : 4;
    if (form == MPM_FORM_FP32) {  // the autotuner's choice on the honeycomb batch
        c->gather_batch = 2;
        c->pass_block = 128;
    }
    c->nspec = nspec;
    cudaGetDevice(&c->device);
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device);
    if (c->sm_count <= 0) c->sm_count = 152;
    if (!cells_attrs<double>() || !cells_attrs<float>() || !pass2_staged_attrs() || !pairs_attr<128>() ||
        !pairs_attr<256>() || !pairs_attr<512>()) {
        cudaGetLastError();
        delete c;
        return MPM_ERR_DEVICE;
    }
    // per-specimen geometry, nodes and cell keys numbered one specimen after the other
    std::vector<double> tab;
    c->geoms.resize(nspec);
    unsigned key_off = 0;
    long long node_off = 0;
    for (int s = 0; s < nspec; ++s) {
        const mpm_grid_desc& gd = grids[s];
        Geom& g = c->geoms[s];
        memset(&g, 0, sizeof(g));
        long long ks = 1, ns = 1;
        for (int a = 0; a < 3; ++a) {
            // d3_Length_Cell = d3Length_Grid / dvec3(i3Cells)
            g.h[a] = gd.length[a] / (double)gd.cells[a];
            g.inv_h[a] = 1.0 / g.h[a];
            set_float_geometry(g, a);
            g.nn[a] = gd.cells[a] + 1;
            g.kd[a] = gd.cells[a] + 2;
            ks *= g.kd[a];
            ns *= g.nn[a];
            // padded node coordinate table: entry n+1 for node n in [-1, nn], (i*L)/cells
            g.xoff[a] = (int)tab.size();
            for (int i = -1; i <= g.nn[a]; ++i) tab.push_back(i * gd.length[a] / gd.cells[a]);
        }
        g.key_off = key_off;
        g.node_off = node_off;
        key_off += (unsigned)ks;
        node_off += ns;
        if (s == 0)
            for (int a = 0; a < 3; ++a) {
                c->length[a] = gd.length[a];
                c->cells[a] = gd.cells[a];
            }
    }
    c->nn = node_off;
    int rc = MPM_OK;
    auto bail = [&](int code) {
        mpm_destroy(c);
        return code;
    };
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(MPM_ERR_CUDA);
    c->own_stream = true;
    if ((rc = ensure(c, c->xtab, tab.size() * 8))) return bail(rc);
    if (cudaMemcpy(c->xtab.p, tab.data(), tab.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(MPM_ERR_CUDA);
    for (Geom& g : c->geoms) {
        g.key_max = key_off;
        g.n_nodes = node_off;
        g.xtab = (const double*)c->xtab.p;
        g.nspec = nspec;
    }
    if (nspec > 1) {
        if ((rc = ensure(c, c->geom_tab, sizeof(Geom) * nspec))) return bail(rc);
        for (Geom& g : c->geoms) g.tab = (const Geom*)c->geom_tab.p;
        if (cudaMemcpy(c->geom_tab.p, c->geoms.data(), sizeof(Geom) * nspec, cudaMemcpyHostToDevice) != cudaSuccess)
            return bail(MPM_ERR_CUDA);
    }
    c->g = c->geoms[0];
    Geom& g = c->g;
    if ((rc = ensure(c, c->err_word, 4))) return bail(rc);
    cudaMemset(c->err_word.p, 0, 4);
    if (cudaMallocHost((void**)&c->h_err, sizeof(unsigned)) != cudaSuccess) return bail(MPM_ERR_CUDA);
    const size_t t = c->tsize, nn = (size_t)c->nn;
    struct {
        DevBuf* b;
        size_t bytes;
    } plan[] = {{&c->g_acc, 8 * nn * t},   {&c->g_vel, 3 * nn * t},
                {&c->g_ftemp, 3 * nn * t}, {&c->g_mg, 3 * nn * t},
                {&c->g_state, nn * 4},     {&c->g_fixed, nn},        {&c->g_friction, nn * 8},
                {&c->g_ratio, 8 * nn * t}, {&c->g_q, 4 * nn * t},    {&c->g_owner, 3 * nn * 4},
                {&c->g_nowner, nn * 4},    {&c->g_need, nn * 4},     {&c->g_list, nn * 4},
                {&c->g_count, 4},          {&c->alist, nn * 4},       {&c->acount, 4},
                // per-cell particle ranges: the FP64 form's exact contact gather only
                {&c->cstart, c->form == MPM_FORM_FP64 ? (size_t)g.key_max * 4 : 0},
                {&c->cend, c->form == MPM_FORM_FP64 ? (size_t)g.key_max * 4 : 0}};
    for (auto& e : plan) {
        if ((rc = ensure(c, *e.b, e.bytes))) return bail(rc);
        if (cudaMemset(e.b->p, 0, e.bytes) != cudaSuccess) return bail(MPM_ERR_CUDA);
    }
    *out = c;
    return MPM_OK;
}

int mpm_batch_info(const mpm_ctx* c, int64_t* node_offsets, int32_t* nspec) {
    if (!c) return MPM_ERR_ARG;
    if (nspec) *nspec = c->nspec;
    if (node_offsets) {
        for (int s = 0; s < c->nspec; ++s) node_offsets[s] = c->geoms[s].node_off;
        node_offsets[c->nspec] = c->nn;
    }
    return MPM_OK;
}

void mpm_destroy(mpm_ctx* c) {
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto& r : c->prof_pending) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    for (auto e : c->ev_pool) cudaEventDestroy(e);
    for (DevBuf* b : c->all)
        if (b->p) cudaFree(b->p);
    if (c->h_err) cudaFreeHost(c->h_err);
    if (c->h_sim) cudaFreeHost(c->h_sim);
    graph_reset(c);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    for (auto e : c->xfer_ev)
        if (e) cudaEventDestroy(e);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    delete c;
}

const char* mpm_last_error(const mpm_ctx* c) { return c ? c->err.c_str() : "null context"; }

int mpm_set_stream(mpm_ctx* c, void* stream) {
    graph_reset(c);
    if (!c) return MPM_ERR_ARG;
    CK(cudaStreamSynchronize(c->stream));
    if (c->own_stream) cudaStreamDestroy(c->stream);
    c->own_stream = false;
    c->stream = (cudaStream_t)stream;
    return MPM_OK;
}

int mpm_set_option(mpm_ctx* c, int key, double value) {
    graph_reset(c);
    if (!c) return MPM_ERR_ARG;
    switch (key) {
        case MPM_OPT_FLOOR_FRICTION: c->floor_friction = value != 0.0; return MPM_OK;
        case MPM_OPT_PROFILE: c->profile = value != 0.0; return MPM_OK;
        case MPM_OPT_P2G_REDUCE:
            if (!(value >= 0.0 && value <= 6.0) || value != (double)(int)value)
                return fail(c, MPM_ERR_ARG, "P2G mode must be 0 to 6");
            if (value >= 5.0 && c->form != MPM_FORM_FP32)
                return fail(c, MPM_ERR_ARG, "P2G modes 5 and 6 are built for the FP32 form");
            c->p2g_reduce = (int)value;
            return MPM_OK;
        case MPM_OPT_GRAPH:
            c->use_graph = value != 0.0;
            return MPM_OK;
        case MPM_OPT_LARGE_STRAIN:
            if (value != 0.0 && value != 1.0) return fail(c, MPM_ERR_ARG, "large strain must be 0 or 1");
            if (value != 0.0 && c->form != MPM_FORM_FP64)
                return fail(c, MPM_ERR_ARG, "the large-strain pass 2 is built for the FP64 form");
            c->large_strain = value != 0.0;
            return MPM_OK;
        case MPM_OPT_SURROGATE_GUARD:
            if (!(value >= 0.0 && value < 1.0)) return fail(c, MPM_ERR_ARG, "guard tolerance must be in [0, 1)");
            c->sg_guard = (float)value;
            return MPM_OK;
        case MPM_OPT_FP64_FALLBACK:
            if (value != 0.0 && value != 1.0) return fail(c, MPM_ERR_ARG, "FP64 fallback must be 0 or 1");
            c->fp64_fallback = value != 0.0;
            return MPM_OK;
        case MPM_OPT_CELL_SORT:
            if (value != 0.0 && value != 1.0) return fail(c, MPM_ERR_ARG, "cell sort must be 0 or 1");
            c->cell_sort = value != 0.0;
            return MPM_OK;
        case MPM_OPT_REORDER:
            if (!(value >= -1.0 && value < 2147483647.0) || value != (double)(long long)value)
                return fail(c, MPM_ERR_ARG, "reorder interval must be -1, 0 or a step count");
            c->reorder_interval = (int)value;
            if (c->reorder_interval < 0) c->reorder_pending = false;
            return MPM_OK;
        case MPM_OPT_GATHER:
            if (value != 0.0 && value != 1.0 && value != 2.0)
                return fail(c, MPM_ERR_ARG, "pass-2 mode must be 0, 1 or 2");
            if (value == 2.0 && c->form != MPM_FORM_FP32)
                return fail(c, MPM_ERR_ARG, "the staged pass 2 is built for the FP32 form");
            c->gather_batch = (int)value;
            return MPM_OK;
        case MPM_OPT_PASS1_CORNERS:
            if (value != 1.0 && value != 2.0 && value != 4.0)
                return fail(c, MPM_ERR_ARG, "pass-1 corners per thread must be 1, 2 or 4");
            c->pass1_corners = (int)value;
            return MPM_OK;
        case MPM_OPT_P2G_BLOCK:
        case MPM_OPT_PASS_BLOCK:
        case MPM_OPT_PASS1_BLOCK: {
            int b = (int)value;
            if (b != 128 && b != 256 && b != 512) return fail(c, MPM_ERR_ARG, "block size must be 128, 256 or 512");
            (key == MPM_OPT_P2G_BLOCK ? c->p2g_block : key == MPM_OPT_PASS_BLOCK ? c->pass_block : c->pass1_block) = b;
            return MPM_OK;
        }
        default: return fail(c, MPM_ERR_ARG, "unknown option %d", key);
    }
}

int mpm_upload_materials(mpm_ctx* c, const mpm_material* m, int32_t n) {
    graph_reset(c);
    if (!c || n < 0 || (n > 0 && !m)) return c ? fail(c, MPM_ERR_ARG, "bad material table") : MPM_ERR_ARG;
    std::vector<MatConst> mc((size_t)std::max(1, n));
    for (int i = 0; i < n; ++i) {
        MatConst& k = mc[i];
        memset(&k, 0, sizeof(k));
        const double E = m[i].E, nu = m[i].nu;
        k.type = m[i].type == MPM_MAT_ELASTIC ? 0 : (m[i].type == MPM_MAT_VONMISESHARDENING ? 4 : 3);
        k.E = E;
        k.nu = nu;
        k.Y = m[i].yield;
        k.C0 = m[i].C0;
        k.C1 = m[i].C1;
        // the reference's own expressions (…_Elastic.cpp:9, …_PerfectlyPlastic.cpp:13,43,64, …_VonMisesHardening.cpp:87)
        k.C = E / (1.0 + nu) / (1.0 - 2.0 * nu);
        k.one_m_nu = 1.0 - nu;
        k.half_m_nu = 0.5 - nu;
        k.G = 0.5 * E / (1.0 + nu);
        k.k0 = m[i].yield / std::sqrt(3.0);
        k.s23C1 = std::sqrt(2.0 / 3.0) * m[i].C1;
        k.inv_E = 1.0 / E;
        k.nu_over_E = nu / E;
        k.inv_G = 1.0 / k.G;
        set_float_constants(k);
    }
    c->mats_host = mc;
    c->sg_mats = 0;
    if (c->net) {
        const MatConst& nm = net_material(c->net);
        for (int i = 0; i < n && i < 32; ++i)
            if (mc[i].type == 4 && mc[i].E == nm.E && mc[i].nu == nm.nu && mc[i].Y == nm.Y && mc[i].C0 == nm.C0 &&
                mc[i].C1 == nm.C1)
                c->sg_mats |= 1u << i;
    }
    int rc = ensure(c, c->mats, mc.size() * sizeof(MatConst));
    if (rc) return rc;
    CK(cudaMemcpyAsync(c->mats.p, mc.data(), mc.size() * sizeof(MatConst), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->nmat = n;
    return MPM_OK;
}

int mpm_upload_particles(mpm_ctx* c, const mpm_particles* p, int64_t n) {
    graph_reset(c);
    if (!c) return MPM_ERR_ARG;
    if (!p || n < 0 || n >= 0x7fffffffLL) return fail(c, MPM_ERR_ARG, "bad particle upload (n=%lld)", (long long)n);
    const bool f64 = c->form == MPM_FORM_FP64;
    int rc;
    if (c->nspec > 1) {
        // specimen ids checked and narrowed on the device (into the staging
        // buffer, then into place once all are valid: a bad upload changes nothing)
        if (!p->specimen && n > 0) return fail(c, MPM_ERR_ARG, "a batch of specimens needs the specimen of each particle");
        const size_t in_bytes = ((size_t)std::max<int64_t>(1, n) * 4 + 15) / 16 * 16;
        if ((rc = ensure(c, c->staging, in_bytes + (size_t)std::max<int64_t>(1, n) * 2 + 4))) return rc;
        unsigned char* stg = (unsigned char*)c->staging.p;
        unsigned* bad = (unsigned*)(stg + in_bytes + (size_t)std::max<int64_t>(1, n) * 2);
        CK(cudaMemsetAsync(bad, 0xff, 4, c->stream));
        if (n > 0) {
            CK(cudaMemcpyAsync(stg, p->specimen, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
            LAUNCH("fill", k_specimen_ids, blocks_for(n), NTHREADS, (const int32_t*)stg, (long long)n, c->nspec,
                   (uint16_t*)(stg + in_bytes), bad);
        }
        CK(cudaMemcpyAsync(c->h_err, bad, 4, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        if (*c->h_err != 0xffffffffu) {
            const long long i = *c->h_err;
            return fail(c, MPM_ERR_ARG, "particle %lld: specimen %d out of range", i, p->specimen[i]);
        }
        if ((rc = ensure(c, c->sid, (size_t)std::max<int64_t>(1, n) * 2))) return rc;
        if (n > 0)
            CK(cudaMemcpyAsync(c->sid.p, stg + in_bytes, (size_t)n * 2, cudaMemcpyDeviceToDevice, c->stream));
    }
    rc = alloc_particles(c, n);
    if (rc) return rc;
    c->n = n;
    struct {
        DevBuf* b;
        const double* h;
        int k;
        bool fp64;
        double def;
    } fields[] = {{&c->pos, p->pos, 3, true, 0.0},
                  {&c->vel, p->vel, 3, f64, 0.0},
                  {&c->fext, p->fext, 3, f64, 0.0},
                  {&c->mass, p->mass, 1, f64, 0.0},
                  {&c->vol, p->vol, 1, f64, 0.0},
                  {&c->vol0, p->vol0, 1, f64, 0.0},
                  {&c->stress, p->stress, 6, f64, 0.0},
                  {&c->strain, p->strain, 6, f64, 0.0},
                  {&c->eps_p, p->eps_p, 6, f64, 0.0},
                  {&c->e_strain, p->e_strain, 1, true, 0.0},
                  {&c->e_strain_max, p->e_strain_max, 1, true, 0.0},
                  {&c->e_strain_ti, p->e_strain_ti, 1, true, 0.0},
                  {&c->e_plastic, p->e_plastic, 1, true, 0.0},
                  {&c->backstress, p->backstress, 1, f64, 0.0},
                  {&c->mp_mg, p->mp_mass_gradient, 3, f64, 0.0},
                  {&c->strain_rate, p->strain_rate, 6, f64, 0.0}};
    if ((rc = xfer_ready(c))) return rc;
    int fi = 0;
    for (auto& f : fields)
        if ((rc = upload_field_pipelined(c, f.h ? fi++ : 0, *f.b, f.h, n, f.k, f.fp64, f.def))) return rc;
    if (p->F) {
        if ((rc = upload_field_pipelined(c, fi++, c->F, p->F, n, 9, f64, 0.0, f64 ? 0 : 1))) return rc;
    } else if (n > 0) {
        if (f64)
            LAUNCH("fill", k_identity9, blocks_for(9 * n), NTHREADS, c->F.p, (long long)n, 1);
        else
            CK(cudaMemsetAsync(c->F.p, 0, (size_t)n * 9 * sizeof(float), c->stream));  // H = F - I = 0
    }
    if (f64) {  // the elastic deformation gradient, identity unless given
        if (p->F_elastic) {
            if ((rc = upload_field(c, c->Fe, p->F_elastic, n, 9, true, 0.0))) return rc;
        } else if (n > 0) {
            LAUNCH("fill", k_identity9, blocks_for(9 * n), NTHREADS, c->Fe.p, (long long)n, 1);
        }
    }
    if (n > 0) {
        if (p->material)
            CK(cudaMemcpyAsync(c->material.p, p->material, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
        else
            CK(cudaMemsetAsync(c->material.p, 0, (size_t)n * 4, c->stream));
        if (p->pflags) {
            CK(cudaMemcpyAsync(c->pflags.p, p->pflags, (size_t)n, cudaMemcpyHostToDevice, c->stream));
            LAUNCH("fill", k_clear_flag, blocks_for(n), NTHREADS, (uint8_t*)c->pflags.p, (long long)n,
                   (uint8_t)PF_IN_DC);
        } else {
            CK(cudaMemsetAsync(c->pflags.p, 0, (size_t)n, c->stream));
        }
        if (p->dc_mult)
            CK(cudaMemcpyAsync(c->dc_mult.p, p->dc_mult, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
        else
            LAUNCH("fill", k_fill<float>, blocks_for(n), NTHREADS, (float*)c->dc_mult.p, (long long)n, 1.0f);
        if (c->ndc > 0)
            LAUNCH("fill", k_mark_dc, blocks_for(c->ndc), NTHREADS, (const unsigned*)c->dclist.p, c->ndc,
                   (uint8_t*)c->pflags.p);
    }
    // the boundary work counts from this upload on
    if ((rc = ensure(c, c->work_acc, 2 * sizeof(double)))) return rc;
    CK(cudaMemsetAsync(c->work_acc.p, 0, 2 * sizeof(double), c->stream));
    // the surface particles (b_Surface) as a list, for the contact kernels
    if ((rc = ensure(c, c->surf, (size_t)std::max<long long>(1, n) * 4))) return rc;
    CK(cudaMemsetAsync(c->g_count.p, 0, 4, c->stream));
    if (n > 0)
        LAUNCH("fill", k_compact_flag, blocks_for(n), NTHREADS, (const uint8_t*)c->pflags.p, (long long)n,
               (uint8_t)MPM_PF_SURFACE, (unsigned*)c->surf.p, (unsigned*)c->g_count.p);
    CK(cudaMemcpyAsync(c->h_err, c->g_count.p, 4, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    c->nsurf = (int)*c->h_err;
    c->have_particles = true;
    c->keys_valid = false;
    c->have_orig = false;  // the upload is in the caller's order
    c->reorder_pending = c->form == MPM_FORM_FP32 && c->reorder_interval >= 0;
    c->last_perm = c->last_skeys = nullptr;
    return MPM_OK;
}

int mpm_upload_dc_list(mpm_ctx* c, const uint32_t* idx, int64_t n) {
    graph_reset(c);
    if (!c) return MPM_ERR_ARG;
    if (n < 0 || (n > 0 && !idx)) return fail(c, MPM_ERR_ARG, "bad displacement-control list");
    if (!c->have_particles && n > 0) return fail(c, MPM_ERR_STATE, "upload particles before the dc list");
    std::vector<uint32_t> sorted(idx, idx + n);
    std::sort(sorted.begin(), sorted.end());
    for (int64_t i = 0; i < n; ++i) {
        if (sorted[i] >= (uint64_t)c->n) return fail(c, MPM_ERR_ARG, "dc index %u out of range", sorted[i]);
        if (i > 0 && sorted[i] == sorted[i - 1]) return fail(c, MPM_ERR_ARG, "duplicate dc index %u", sorted[i]);
    }
    int rc = ensure(c, c->dclist, (size_t)std::max<int64_t>(1, n) * 4);
    if (rc) return rc;
    if (c->n > 0)
        LAUNCH("fill", k_clear_flag, blocks_for(c->n), NTHREADS, (uint8_t*)c->pflags.p, c->n, (uint8_t)PF_IN_DC);
    if (n > 0) {
        CK(cudaMemcpyAsync(c->dclist.p, idx, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
        if (c->have_orig) {  // caller's indices -> slots
            if ((rc = ensure(c, c->ptmp, (size_t)c->n * 4))) return rc;
            LAUNCH("fill", k_invert, blocks_for(c->n), NTHREADS, (const unsigned*)c->orig.p, (unsigned*)c->ptmp.p, c->n);
            LAUNCH("fill", k_remap_list, blocks_for(n), NTHREADS, (unsigned*)c->dclist.p, (long long)n,
                   (const unsigned*)c->ptmp.p);
        }
        LAUNCH("fill", k_mark_dc, blocks_for(n), NTHREADS, (const unsigned*)c->dclist.p, (int)n,
               (uint8_t*)c->pflags.p);
    }
    CK(cudaStreamSynchronize(c->stream));
    c->ndc = (int)n;
    return MPM_OK;
}

int mpm_upload_nodes(mpm_ctx* c, const mpm_nodes* nd) {
    graph_reset(c);
    if (!c) return MPM_ERR_ARG;
    if (!nd) return fail(c, MPM_ERR_ARG, "null node view");
    const long long nn = c->nn;
    const bool f64 = c->form == MPM_FORM_FP64;
    int rc;
    if (nd->fixed)
        CK(cudaMemcpyAsync(c->g_fixed.p, nd->fixed, (size_t)nn, cudaMemcpyHostToDevice, c->stream));
    if (nd->friction)
        CK(cudaMemcpyAsync(c->g_friction.p, nd->friction, (size_t)nn * 8, cudaMemcpyHostToDevice, c->stream));
    struct {
        DevBuf* b;
        const double* h;
        int k;
        int acc;  // component of the accumulator record, or -1
    } fields[] = {{&c->g_acc, nd->mass, 1, 0},   {&c->g_acc, nd->mom, 3, 1},
                  {&c->g_vel, nd->vel, 3, -1},   {&c->g_acc, nd->force, 3, 4},
                  {&c->g_ftemp, nd->force_temp, 3, -1}, {&c->g_mg, nd->mass_gradient, 3, -1}};
    for (auto& f : fields)
        if (f.h && (rc = upload_field(c, *f.b, f.h, nn, f.k, f64, 0.0, 0, f.acc))) return rc;
    if (nd->state) {
        int rc2 = ensure(c, c->staging, (size_t)nn);
        if (rc2) return rc2;
        CK(cudaMemcpyAsync(c->staging.p, nd->state, (size_t)nn, cudaMemcpyHostToDevice, c->stream));
        LAUNCH("unpack", k_state_u8_to_u32, blocks_for(nn), NTHREADS, (const uint8_t*)c->staging.p,
               (unsigned*)c->g_state.p, nn);
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    c->have_nodes = true;
    c->have_alist = false;
    c->grid_dirty = true;
    return MPM_OK;
}

int mpm_set_timeline(mpm_ctx* c, const double* t, const double* v3, int32_t n) {
    graph_reset(c);
    if (!c) return MPM_ERR_ARG;
    if (n < 0 || (n > 0 && (!t || !v3))) return fail(c, MPM_ERR_ARG, "bad timeline");
    c->tl_t.assign(t, t + n);
    c->tl_v.assign(v3, v3 + 3 * (size_t)n);
    if (n > 0) {  // device copy (t[n], v[3n]) for the step graph's clock
        int rc = ensure(c, c->tl_dev, (size_t)4 * n * 8);
        if (rc) return rc;
        CK(cudaMemcpy(c->tl_dev.p, t, (size_t)n * 8, cudaMemcpyHostToDevice));
        CK(cudaMemcpy((double*)c->tl_dev.p + n, v3, (size_t)3 * n * 8, cudaMemcpyHostToDevice));
    }
    return MPM_OK;
}

int mpm_set_sim(mpm_ctx* c, const mpm_sim* s) {
    if (!c || !s) return MPM_ERR_ARG;
    // the step graph bakes in the mass threshold and the damping; time and
    // step count reach it through the device clock, set at every replay
    if (s->mass_min != c->sim.mass_min || s->damping != c->sim.damping) graph_reset(c);
    c->sim = *s;
    return MPM_OK;
}

int mpm_get_sim(const mpm_ctx* c, mpm_sim* s) {
    if (!c || !s) return MPM_ERR_ARG;
    *s = c->sim;
    return MPM_OK;
}

int mpm_download_particles(mpm_ctx* c, mpm_particles* p) {
    if (!c || !p) return MPM_ERR_ARG;
    const long long n = c->n;
    const bool f64 = c->form == MPM_FORM_FP64;
    int rc;
    struct {
        DevBuf* b;
        double* h;
        int k;
        bool fp64;
    } fields[] = {{&c->pos, p->pos, 3, true},
                  {&c->vel, p->vel, 3, f64},
                  {&c->fext, p->fext, 3, f64},
                  {&c->mass, p->mass, 1, f64},
                  {&c->vol, p->vol, 1, f64},
                  {&c->vol0, p->vol0, 1, f64},
                  {&c->F, p->F, 9, f64},
                  {&c->stress, p->stress, 6, f64},
                  {&c->strain, p->strain, 6, f64},
                  {&c->eps_p, p->eps_p, 6, f64},
                  {&c->e_strain, p->e_strain, 1, true},
                  {&c->e_strain_max, p->e_strain_max, 1, true},
                  {&c->e_strain_ti, p->e_strain_ti, 1, true},
                  {&c->e_plastic, p->e_plastic, 1, true},
                  {&c->backstress, p->backstress, 1, f64},
                  {&c->mp_mg, p->mp_mass_gradient, 3, f64},
                  {&c->strain_rate, p->strain_rate, 6, f64},
                  {&c->Fe, f64 ? p->F_elastic : nullptr, 9, true}};
    if ((rc = xfer_ready(c))) return rc;
    int fi = 0;
    for (auto& f : fields) {
        if (!f.h) continue;
        const int shift = (f.b == &c->F && !f64) ? 1 : 0;
        if ((rc = download_field_pipelined(c, fi++, *f.b, f.h, n, f.k, f.fp64, shift))) return rc;
    }
    CK(cudaStreamSynchronize(c->copy_stream));
    CK(cudaStreamSynchronize(c->stream));
    if (!f64 && p->F_elastic)  // the FP32 form has no large-strain pass: the identity
        for (long long i = 0; i < n; ++i)
            for (int k = 0; k < 9; ++k) p->F_elastic[9 * i + k] = (k == 0 || k == 4 || k == 8) ? 1.0 : 0.0;
    if (n > 0) {
        // in the caller's order: through the staging buffer when the slots are in cell order
        auto get = [&](void* host, const DevBuf& b, int es) -> int {
            if (!host) return MPM_OK;
            if (!c->have_orig) {
                CK(cudaMemcpyAsync(host, b.p, (size_t)n * es, cudaMemcpyDeviceToHost, c->stream));
                return MPM_OK;
            }
            int r = ensure(c, c->staging, (size_t)n * 8);
            if (r) return r;
            if (es == 4)
                LAUNCH("pack", k_scatter_orig<4>, blocks_for(n), NTHREADS, b.p, c->staging.p, (const unsigned*)c->orig.p, n);
            else
                LAUNCH("pack", k_scatter_orig<1>, blocks_for(n), NTHREADS, b.p, c->staging.p, (const unsigned*)c->orig.p, n);
            CK(cudaMemcpyAsync(host, c->staging.p, (size_t)n * es, cudaMemcpyDeviceToHost, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            return MPM_OK;
        };
        if ((rc = get(p->material, c->material, 4)) || (rc = get(p->pflags, c->pflags, 1)) ||
            (rc = get(p->dc_mult, c->dc_mult, 4)))
            return rc;
    }
    CK(cudaStreamSynchronize(c->stream));
    if (p->pflags)
        for (long long i = 0; i < n; ++i) p->pflags[i] &= (uint8_t)~PF_IN_DC;
    return check_device_error(c);
}

int mpm_download_nodes(mpm_ctx* c, mpm_nodes* nd) {
    if (!c || !nd) return MPM_ERR_ARG;
    const long long nn = c->nn;
    const bool f64 = c->form == MPM_FORM_FP64;
    int rc;
    struct {
        DevBuf* b;
        double* h;
        int k;
        int acc;  // component of the accumulator record, or -1
    } fields[] = {{&c->g_acc, nd->mass, 1, 0},   {&c->g_acc, nd->mom, 3, 1},
                  {&c->g_vel, nd->vel, 3, -1},   {&c->g_acc, nd->force, 3, 4},
                  {&c->g_ftemp, nd->force_temp, 3, -1}, {&c->g_mg, nd->mass_gradient, 3, -1}};
    for (auto& f : fields) {
        if (!f.h) continue;
        if ((rc = download_field(c, *f.b, f.h, nn, f.k, f64, 0, false, f.acc))) return rc;
        CK(cudaStreamSynchronize(c->stream));
    }
    if (nd->fixed) CK(cudaMemcpyAsync(nd->fixed, c->g_fixed.p, (size_t)nn, cudaMemcpyDeviceToHost, c->stream));
    if (nd->friction)
        CK(cudaMemcpyAsync(nd->friction, c->g_friction.p, (size_t)nn * 8, cudaMemcpyDeviceToHost, c->stream));
    if (nd->state) {
        if ((rc = ensure(c, c->staging, (size_t)nn))) return rc;
        LAUNCH("pack", k_state_u32_to_u8, blocks_for(nn), NTHREADS, (const unsigned*)c->g_state.p,
               (uint8_t*)c->staging.p, nn);
        CK(cudaMemcpyAsync(nd->state, c->staging.p, (size_t)nn, cudaMemcpyDeviceToHost, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    return check_device_error(c);
}

int mpm_advance(mpm_ctx* c, int32_t nsteps, double dt, int contact) {
    if (!c) return MPM_ERR_ARG;
    if (nsteps < 0 || !(dt > 0.0) || !std::isfinite(dt)) return fail(c, MPM_ERR_ARG, "bad step request");
    if (!c->have_particles) return fail(c, MPM_ERR_STATE, "no particles uploaded");
    if (c->nmat <= 0 && c->n > 0) return fail(c, MPM_ERR_STATE, "no materials uploaded");
    return advance_graph(c, nsteps, dt, contact ? 1 : 0);
}

int mpm_run(mpm_ctx* c, double dt_total, int contact, int* done) {
    if (!c) return MPM_ERR_ARG;
    if (!(dt_total >= 0.0)) return fail(c, MPM_ERR_ARG, "bad dt_total");
    // …MPLocks.cpp:449-458: the step sizes of the chunking loop, run in runs of
    // equal size (so the full-size steps can replay the step graph)
    double acc = 0.0;
    double run_dt = 0.0;
    int run_len = 0;
    while (acc < dt_total) {
        double dt = c->sim.dt_max;
        if (c->sim.dt_max > (dt_total - acc)) dt = dt_total - acc;
        acc += dt;
        if (run_len > 0 && dt != run_dt) {
            int rc = mpm_advance(c, run_len, run_dt, contact);
            if (rc) return rc;
            run_len = 0;
        }
        run_dt = dt;
        ++run_len;
    }
    if (run_len > 0) {
        int rc = mpm_advance(c, run_len, run_dt, contact);
        if (rc) return rc;
    }
    int rc = mpm_synchronize(c);
    if (rc) return rc;
    if (done) *done = c->sim.time < c->sim.time_end ? 0 : 1;
    return MPM_OK;
}

int mpm_synchronize(mpm_ctx* c) {
    if (!c) return MPM_ERR_ARG;
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaGetLastError());
    return check_device_error(c);
}

int mpm_advance_timed(mpm_ctx* c, int32_t nsteps, double dt, int contact, float* ms) {
    if (!c) return MPM_ERR_ARG;
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    CK(cudaEventRecord(a, c->stream));
    int rc = mpm_advance(c, nsteps, dt, contact);
    cudaEventRecord(b, c->stream);
    cudaEventSynchronize(b);
    float t = 0.f;
    cudaEventElapsedTime(&t, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (ms) *ms = t;
    if (rc) return rc;
    return check_device_error(c);
}

int mpm_cell_order(mpm_ctx* c, uint32_t* keys, uint32_t* sorted_order, int64_t n) {
    if (!c) return MPM_ERR_ARG;
    if (n != c->n) return fail(c, MPM_ERR_ARG, "n = %lld, engine holds %lld particles", (long long)n, c->n);
    if (!c->last_skeys && n > 0) return fail(c, MPM_ERR_STATE, "no step has run yet");
    std::vector<uint32_t> perm((size_t)std::max<int64_t>(1, n)), skeys((size_t)std::max<int64_t>(1, n));
    bool unsorted = false;  // a step without the sort: slot keys in storage order
    if (n > 0) {
        if (c->last_perm)
            CK(cudaMemcpyAsync(perm.data(), c->last_perm, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
        else
            unsorted = true;
        CK(cudaMemcpyAsync(skeys.data(), c->last_skeys, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    if (unsorted) {  // the stable order of the slots by key
        for (int64_t s = 0; s < n; ++s) perm[s] = (uint32_t)s;
        std::stable_sort(perm.begin(), perm.begin() + n, [&](uint32_t a, uint32_t b) { return skeys[a] < skeys[b]; });
        std::vector<uint32_t> sk((size_t)n);
        for (int64_t s = 0; s < n; ++s) sk[s] = skeys[perm[s]];
        skeys.swap(sk);
    }
    // the last step's key of slot perm[s] is its sorted key skeys[s]
    if (!c->have_orig) {
        if (keys)
            for (int64_t s = 0; s < n; ++s) keys[perm[s]] = skeys[s];
        if (sorted_order && n > 0) memcpy(sorted_order, perm.data(), (size_t)n * 4);
        return MPM_OK;
    }
    // slots in cell order: keys by the caller's index, and the stable order of those indices by key
    std::vector<uint32_t> orig((size_t)n), k((size_t)n);
    CK(cudaMemcpy(orig.data(), c->orig.p, (size_t)n * 4, cudaMemcpyDeviceToHost));
    for (int64_t s = 0; s < n; ++s) k[orig[perm[s]]] = skeys[s];
    if (keys) memcpy(keys, k.data(), (size_t)n * 4);
    if (sorted_order) {
        for (int64_t i = 0; i < n; ++i) sorted_order[i] = (uint32_t)i;
        std::stable_sort(sorted_order, sorted_order + n, [&](uint32_t a, uint32_t b) { return k[a] < k[b]; });
    }
    return MPM_OK;
}

int mpm_upload_monitor_mask(mpm_ctx* c, const uint8_t* mask, int64_t n) {
    graph_reset(c);
    if (!c) return MPM_ERR_ARG;
    if (n != c->n || (n > 0 && !mask)) return fail(c, MPM_ERR_ARG, "monitor mask must have one entry per particle");
    int rc = ensure(c, c->mon_mask, (size_t)std::max<int64_t>(1, n));
    if (rc) return rc;
    if (n > 0) CK(cudaMemcpyAsync(c->mon_mask.p, mask, (size_t)n, cudaMemcpyHostToDevice, c->stream));
    if (n > 0 && c->have_orig) {  // slot s takes the caller's entry orig[s]
        if ((rc = ensure(c, c->ptmp, (size_t)n))) return rc;
        LAUNCH("fill", k_permute<1>, blocks_for(n), NTHREADS, c->mon_mask.p, c->ptmp.p, (const unsigned*)c->orig.p, n, 1);
        CK(cudaMemcpyAsync(c->mon_mask.p, c->ptmp.p, (size_t)n, cudaMemcpyDeviceToDevice, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    c->have_mon = true;
    return MPM_OK;
}

int mpm_monitors_read(mpm_ctx* c, mpm_monitors* out) {
    if (!c || !out) return MPM_ERR_ARG;
    if (!c->have_mon && c->n > 0) return fail(c, MPM_ERR_STATE, "no monitor mask uploaded");
    int rc = ensure(c, c->mon_acc, MON_SLOTS * 8);
    if (rc) return rc;
    CK(cudaMemsetAsync(c->mon_acc.p, 0, MON_SLOTS * 8, c->stream));
    double* acc = (double*)c->mon_acc.p;
    const uint8_t* mask = (const uint8_t*)c->mon_mask.p;
    if (c->form == MPM_FORM_FP64) {
        if (c->n > 0) LAUNCH("monitors", k_monitors<double>, blocks_for(c->n), NTHREADS, pview<double>(c), mask, acc);
        LAUNCH("monitors", k_monitor_force<double>, blocks_for(c->nn), NTHREADS, nview<double>(c), acc);
    } else {
        if (c->n > 0) LAUNCH("monitors", k_monitors<float>, blocks_for(c->n), NTHREADS, pview<float>(c), mask, acc);
        LAUNCH("monitors", k_monitor_force<float>, blocks_for(c->nn), NTHREADS, nview<float>(c), acc);
    }
    double a[MON_SLOTS];
    CK(cudaMemcpyAsync(a, c->mon_acc.p, MON_SLOTS * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    int64_t cnt[5];
    memcpy(cnt, &a[24], sizeof(cnt));
    memset(out, 0, sizeof(*out));
    out->time = c->sim.time;
    for (int k = 0; k < 5; ++k) out->count[k] = cnt[k];
    for (int i = 0; i < 3; ++i) {
        out->position_mean[i] = cnt[0] ? a[i] / (double)cnt[0] : 0.0;
        out->momentum[i] = a[3 + i];
        out->stress_mean[i] = cnt[3] ? a[8 + i] / (double)cnt[3] : 0.0;
        out->strain_mean[i] = cnt[3] ? a[11 + i] / (double)cnt[3] : 0.0;
        out->force_sum[i] = a[17 + i];
    }
    out->strain_p_max = a[6];
    out->stress_p_max = a[7];
    out->kinetic = a[14];
    out->strain_energy = a[15];
    out->plastic_energy = a[16];
    double w[2] = {0.0, 0.0};
    if (c->work_acc.p) {
        CK(cudaMemcpyAsync(w, c->work_acc.p, sizeof(w), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    out->platen_work = w[0];
    out->friction_work = w[1];
    return check_device_error(c);
}

int mpm_autotune(mpm_ctx* c, int32_t steps, double dt, int contact, mpm_tune_result* out) {
    graph_reset(c);
    if (!c) return MPM_ERR_ARG;
    if (steps < 1 || !(dt > 0.0)) return fail(c, MPM_ERR_ARG, "bad autotune request");
    if (!c->have_particles) return fail(c, MPM_ERR_STATE, "no particles uploaded");
    if (c->reorder_pending) {  // the trials time the storage order the run will have
        int r0 = reorder(c);
        if (r0) return r0;
    }
    const long long since0 = c->steps_since_reorder;
    // everything a step writes that outlives the step
    DevBuf* state[] = {&c->pos,        &c->vel,      &c->F,          &c->stress,  &c->strain,  &c->eps_p,
                       &c->vol,        &c->e_strain, &c->e_strain_max, &c->e_strain_ti, &c->e_plastic,
                       &c->backstress, &c->mp_mg,    &c->strain_rate, &c->g_acc,   &c->g_vel,
                       &c->g_ftemp,  &c->g_mg,       &c->g_state,     &c->work_acc};
    size_t total = 0;
    for (DevBuf* b : state) total += b->bytes;
    int rc = ensure(c, c->tune_backup, total);
    if (rc) return rc;
    auto copy_all = [&](bool save) -> int {
        size_t off = 0;
        for (DevBuf* b : state) {
            char* bk = (char*)c->tune_backup.p + off;
            if (b->bytes)
                CK(cudaMemcpyAsync(save ? bk : b->p, save ? b->p : bk, b->bytes, cudaMemcpyDeviceToDevice,
                                   c->stream));
            off += b->bytes;
        }
        return MPM_OK;
    };
    if ((rc = copy_all(true))) return rc;
    const mpm_sim sim0 = c->sim;
    const int prof0 = c->profile;
    c->profile = 0;
    // the tuned options: P2G mode, P2G block, pass-1 corners, pass-1 block, pass-2 block, gather mode
    int* opt[6] = {&c->p2g_reduce, &c->p2g_block, &c->pass1_corners, &c->pass1_block, &c->pass_block, &c->gather_batch};
    int old[6], best[6];
    for (int i = 0; i < 6; ++i) old[i] = best[i] = *opt[i];
    double best_ms = 1e300, worst_ms = 0.0;
    int ncand = 0;
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    // one trial: the candidate's options over the best so far, a warm-up step, `steps` timed steps, restore
    auto trial = [&](int i0, int v0, int i1, int v1) -> int {
        for (int i = 0; i < 6; ++i) *opt[i] = best[i];
        *opt[i0] = v0;
        *opt[i1] = v1;
        int r = step(c, dt, contact, false, false);  // the run's steps: not output steps
        if (r == MPM_OK) {
            cudaEventRecord(a, c->stream);
            for (int s = 0; s < steps && r == MPM_OK; ++s) r = step(c, dt, contact, false, false);
            cudaEventRecord(b, c->stream);
        }
        if (r == MPM_OK) {
            cudaEventSynchronize(b);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, a, b);
            const double per = ms / steps;
            ++ncand;
            worst_ms = std::max(worst_ms, per);
            if (per < best_ms) {
                best_ms = per;
                for (int i = 0; i < 6; ++i) best[i] = *opt[i];
            }
        }
        if (copy_all(false) != MPM_OK && r == MPM_OK) r = MPM_ERR_CUDA;
        c->keys_valid = false;  // positions restored: keys are recomputed next step
        c->have_alist = false;
        c->grid_dirty = true;
        c->sim = sim0;
        return r;
    };
    const int blocks[3] = {128, 256, 512}, corners[3] = {1, 2, 4};
    const int p2g_modes = c->form == MPM_FORM_FP32 ? 7 : 5;
    for (int red = 0; red < p2g_modes && rc == MPM_OK; ++red)
        for (int pb = 0; pb < 3 && rc == MPM_OK; ++pb) rc = trial(0, red, 1, blocks[pb]);
    if (best[0] >= 2)
        for (int k = 0; k < 3 && rc == MPM_OK; ++k)
            for (int pb = 0; pb < 3 && rc == MPM_OK; ++pb) rc = trial(2, corners[k], 3, blocks[pb]);
    const int gmodes = c->form == MPM_FORM_FP32 ? 3 : 2;
    for (int qb = 0; qb < 3 && rc == MPM_OK; ++qb)
        for (int gb = 0; gb < gmodes && rc == MPM_OK; ++gb) rc = trial(4, blocks[qb], 5, gb);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    c->steps_since_reorder = since0;
    c->profile = prof0;
    c->sim = sim0;
    if (rc) {
        for (int i = 0; i < 6; ++i) *opt[i] = old[i];
        return rc;
    }
    CK(cudaStreamSynchronize(c->stream));
    for (int i = 0; i < 6; ++i) *opt[i] = best[i];
    if (out) {
        out->p2g_reduce = best[0];
        out->p2g_block = best[1];
        out->pass1_corners = best[2];
        out->pass1_block = best[3];
        out->pass_block = best[4];
        out->gather_batch = best[5];
        out->candidates = ncand;
        out->best_ms_per_step = best_ms;
        out->worst_ms_per_step = worst_ms;
    }
    return check_device_error(c);
}

int mpm_profile_read(mpm_ctx* c, mpm_kernel_stat* out, int32_t max, int32_t* count) {
    if (!c) return MPM_ERR_ARG;
    int rc = prof_resolve(c);
    if (rc) return rc;
    int n = (int)c->prof_names.size();
    if (count) *count = n;
    for (int i = 0; i < n && i < max && out; ++i) {
        memset(out[i].name, 0, sizeof(out[i].name));
        strncpy(out[i].name, c->prof_names[i].c_str(), sizeof(out[i].name) - 1);
        out[i].launches = c->prof_cnt[i];
        out[i].total_ms = c->prof_ms[i];
    }
    return MPM_OK;
}

int mpm_profile_reset(mpm_ctx* c) {
    if (!c) return MPM_ERR_ARG;
    int rc = prof_resolve(c);
    if (rc) return rc;
    std::fill(c->prof_ms.begin(), c->prof_ms.end(), 0.0);
    std::fill(c->prof_cnt.begin(), c->prof_cnt.end(), 0LL);
    return MPM_OK;
}

int mpm_attach_surrogate(mpm_ctx* c, mpm_net* net, double band, double recheck) {
    graph_reset(c);
    if (!c) return MPM_ERR_ARG;
    if (net && c->form != MPM_FORM_FP32) return fail(c, MPM_ERR_ARG, "the return-map network serves the FP32 form");
    if (net && !(band >= 0.0 && band < 10.0 && recheck >= 0.0 && recheck <= 1.0))
        return fail(c, MPM_ERR_ARG, "band must be in [0, 10), recheck in [0, 1]");
    c->net = net;
    c->sg_band = (float)band;
    c->sg_recheck = (float)recheck;
    c->sg_mats = 0;
    if (net) {
        const MatConst& nm = net_material(net);
        for (size_t i = 0; i < c->mats_host.size() && i < (size_t)c->nmat && i < 32; ++i) {
            const MatConst& m = c->mats_host[i];
            if (m.type == 4 && m.E == nm.E && m.nu == nm.nu && m.Y == nm.Y && m.C0 == nm.C0 && m.C1 == nm.C1)
                c->sg_mats |= 1u << i;
        }
        int rc = ensure(c, c->sg_acc, sizeof(SurrogateAcc));
        if (rc) return rc;
        CK(cudaMemsetAsync(c->sg_acc.p, 0, sizeof(SurrogateAcc), c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    return MPM_OK;
}

int mpm_harvest_begin(mpm_ctx* c, float* d_rows, int64_t cap, uint32_t mat_mask, double band) {
    graph_reset(c);
    if (!c) return MPM_ERR_ARG;
    if (!d_rows || cap < 1 || !(band >= 0.0)) return fail(c, MPM_ERR_ARG, "harvest needs rows, cap >= 1, band >= 0");
    int rc = ensure(c, c->hv_count, 64);
    if (rc) return rc;
    CK(cudaMemsetAsync(c->hv_count.p, 0, 4, c->stream));
    c->hv_on = 1;
    c->hv_rows = d_rows;
    c->hv_cap = cap;
    c->hv_mats = mat_mask;
    c->hv_band = (float)band;
    return MPM_OK;
}

int mpm_harvest_end(mpm_ctx* c, int64_t* rows) {
    graph_reset(c);
    if (!c || !rows) return MPM_ERR_ARG;
    *rows = 0;
    if (!c->hv_on) return MPM_OK;
    unsigned h = 0;
    CK(cudaMemcpyAsync(&h, c->hv_count.p, 4, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    *rows = (int64_t)h;
    c->hv_on = 0;
    c->hv_rows = nullptr;
    c->hv_cap = 0;
    return MPM_OK;
}

int mpm_surrogate_stats_read(mpm_ctx* c, mpm_surrogate_stats* out, int reset) {
    if (!c || !out) return MPM_ERR_ARG;
    memset(out, 0, sizeof(*out));
    if (!c->sg_acc.p) return MPM_OK;
    SurrogateAcc h;
    CK(cudaMemcpyAsync(&h, c->sg_acc.p, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    out->queued = (int64_t)h.queued;
    out->band = (int64_t)h.band;
    out->rechecked = (int64_t)h.rechecked;
    out->recheck_rms = h.rechecked ? std::sqrt(h.sq_err / (double)h.rechecked) : 0.0;
    out->recheck_max = h.max_err;
    out->rejected = (int64_t)h.rejected;
    if (reset) {
        CK(cudaMemsetAsync(c->sg_acc.p, 0, sizeof(SurrogateAcc), c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    return MPM_OK;
}

int mpm_launch_count(const mpm_ctx* c, int64_t* count) {
    if (!c || !count) return MPM_ERR_ARG;
    *count = c->launches;
    return MPM_OK;
}

}  // extern "C"
