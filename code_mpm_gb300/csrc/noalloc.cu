// mpm_cell_order_noalloc: cell keys and the stable order by cell of
// caller-provided device positions, computed without allocating memory.
//
// Some hosts of this engine cannot allocate device memory at the moment they
// need the cell order: code running inside a memory pool or arena that owns
// every byte of the device heap, plug-ins whose host framework forbids
// cudaMalloc/cudaFree on its calling thread (for example between the
// framework's own allocation phases), and latency-critical callers for whom
// an allocation (and the implicit device synchronisation of cudaFree) in the
// loop is not acceptable.  This entry point needs nothing from the caller
// except its inputs and outputs: its working memory (the radix sort's
// ping-pong key/value buffers and digit histograms) lives in one file-scope
// __device__ array below, reserved when the library is loaded and held by
// every GPU that loads it until the process exits.
//
// The result is the same as mpm_cell_order() reports for the same positions
// (same kernels, same stable LSD radix sort).
#include <cuda_runtime.h>

#include <mutex>

#include "kernels.cuh"
#include "mpm_gb300.h"
#include "radix_sort.cuh"

using namespace mpm;

namespace {

constexpr long long NA_MAX = MPM_NOALLOC_MAX_PARTICLES;
constexpr long long NA_TILES = (NA_MAX + RS_TILE - 1) / RS_TILE;
// layout (32-bit words): keysA, valsA, keysB, valsB (NA_MAX each), digit counts
// (256 per tile), then one word k_cell_keys may flag a non-finite position in
// (a write-only sink: such a particle already gets the out-of-grid key, and
// the word is never read), padded to 64 words.
constexpr long long NA_WORDS = 4 * NA_MAX + 256 * NA_TILES + 64;

// The scratch: file scope, static storage on every device that loads the library.
__device__ __align__(256) unsigned g_noalloc_scratch[NA_WORDS];

constexpr int NA_MAX_DEVICES = 64;
unsigned* g_scratch_addr[NA_MAX_DEVICES] = {nullptr};
std::mutex g_setup_mutex;

// Once per device, with that device current: the device address of the
// scratch array.  In host code g_noalloc_scratch names a host-side shadow,
// not device memory, so only this address may be handed to kernels.
int scratch_for_current_device(unsigned** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MPM_ERR_CUDA;
    if (dev < 0 || dev >= NA_MAX_DEVICES) return MPM_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return MPM_ERR_CUDA;
        }
        g_scratch_addr[dev] = (unsigned*)p;
    }
    *out = g_scratch_addr[dev];
    return MPM_OK;
}

}  // namespace

extern "C" int mpm_cell_order_noalloc(const mpm_grid_desc* grid, const double* d_pos, int64_t n, uint32_t* d_keys,
                                      uint32_t* d_order, void* stream) {
    if (!grid || n < 0) return MPM_ERR_ARG;
    if (n > NA_MAX) return MPM_ERR_TOO_LARGE;
    if (n == 0) return MPM_OK;
    if (!d_pos || !d_keys || !d_order) return MPM_ERR_ARG;
    Geom g{};
    long long keyspace = 1;
    for (int a = 0; a < 3; ++a) {
        // cells + 2 must fit an int, and the key count a 32-bit key: check each factor before multiplying
        if (!(grid->length[a] > 0.0) || grid->cells[a] < 1 || grid->cells[a] > (1 << 30)) return MPM_ERR_ARG;
        g.h[a] = grid->length[a] / (double)grid->cells[a];
        g.inv_h[a] = 1.0 / g.h[a];
        set_float_geometry(g, a);
        g.nn[a] = grid->cells[a] + 1;
        g.kd[a] = grid->cells[a] + 2;
        keyspace *= (long long)g.kd[a];  // < 2^32 * (2^30 + 2): no overflow
        if (keyspace >= 0xffffffffLL) return MPM_ERR_ARG;
    }
    g.key_max = (unsigned)keyspace;
    // an error left pending by the caller's own work is not this call's to report or to clear
    if (cudaPeekAtLastError() != cudaSuccess) return MPM_ERR_CUDA;
    unsigned* s = nullptr;
    int rc = scratch_for_current_device(&s);
    if (rc) return rc;
    unsigned* keysA = s;
    unsigned* valsA = s + NA_MAX;
    unsigned* keysB = s + 2 * NA_MAX;
    unsigned* valsB = s + 3 * NA_MAX;
    unsigned* counts = s + 4 * NA_MAX;
    unsigned* err = counts + 256 * NA_TILES;
    cudaStream_t st = (cudaStream_t)stream;
    // every scratch word the sort reads is written first by this call (keys and values by k_cell_keys,
    // digit counts by each pass's histogram), so the previous call's contents need no clearing
    const unsigned nb = (unsigned)((n + 255) / 256);
    k_cell_keys<<<nb, 256, 0, st>>>(d_pos, n, g, keysA, valsA, d_keys, err, nullptr, nullptr);
    if (cudaGetLastError() != cudaSuccess) return MPM_ERR_CUDA;
    int bits = 1;
    while (bits < 32 && ((unsigned long long)1 << bits) <= (unsigned long long)g.key_max) ++bits;
    const int nblocks = (int)((n + RS_TILE - 1) / RS_TILE);
    unsigned *kin = keysA, *vin = valsA, *kout = keysB, *vout = valsB;
    for (int shift = 0; shift < bits; shift += 8) {
        k_rs_hist<<<nblocks, RS_THREADS, 0, st>>>(kin, n, shift, counts, nblocks);
        if (cudaGetLastError() != cudaSuccess) return MPM_ERR_CUDA;
        k_rs_scan<<<1, 1024, 0, st>>>(counts, 256 * nblocks);
        if (cudaGetLastError() != cudaSuccess) return MPM_ERR_CUDA;
        k_rs_scatter<<<nblocks, RS_THREADS, 0, st>>>(kin, vin, kout, vout, n, shift, counts, nblocks, nullptr);
        if (cudaGetLastError() != cudaSuccess) return MPM_ERR_CUDA;
        unsigned* t = kin;
        kin = kout;
        kout = t;
        t = vin;
        vin = vout;
        vout = t;
    }
    if (cudaMemcpyAsync(d_order, vin, (size_t)n * sizeof(unsigned), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return MPM_ERR_CUDA;
    return MPM_OK;
}
