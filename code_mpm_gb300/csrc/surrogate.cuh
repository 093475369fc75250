// Internal interface between the engine and the return-map network
// (surrogate.cu): the pieces pass 2 and the step driver need.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

struct mpm_net;

namespace mpm {

// A particle whose return map the network computes: its inputs in physical
// units (stress, R, strain increment), what the finishing kernel needs to
// apply the result (volume, particle index), and the network's outputs.
struct SurrogateQueue {
    float* in;         // cap x 13
    float* out;        // cap x 7
    float* vol;        // cap
    unsigned* pidx;    // cap
    unsigned* count;   // device counter (pass 2 appends)
    long long cap;
};

// Counters of the in-loop use (device, doubles/u64 as laid out here).
struct SurrogateAcc {
    unsigned long long queued, band, rechecked, rejected;
    double sq_err, max_err;  // over rechecks, |dsigma error| / yield
};

// The guard on the network's results: the box of normalised inputs the
// network was trained on, the input scaling, and the tolerance (a fraction
// of k0) of the plasticity checks.  A result outside the guard is replaced by
// the exact map in FP64.
struct SurrogateGuard {
    float in_inv_scale[13];
    float lo[13], hi[13];
    float tol;
};

// Run the network over the queue (device-side count; no host sync).
int net_run_queue(mpm_net* net, const SurrogateQueue& q, cudaStream_t s, unsigned* err);
// The material the network was trained for, and its yield stress.
const MatConst& net_material(const mpm_net* net);
float net_yield(const mpm_net* net);
// The guard of the network's results at tolerance tol (tol <= 0: no guard).
SurrogateGuard net_guard(const mpm_net* net, float tol);

}  // namespace mpm
