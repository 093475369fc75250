/*
 * mpm_gb300.h -- C ABI of the GB300 explicit-MPM engine.
 *
 * The engine replaces one hot path of the reference solver: the classic
 * double-pass (USL) step of
 *   PhysicsEngine::runSimulation_Classic_DoublePass_MPLocks(double)          PhysicsEngine.h:54
 *   PhysicsEngine::runSimulation_Classic_DoublePass_MPLocks_Contact(double)  PhysicsEngine.h:55
 * i.e. reset grid -> find adjacent grid points -> P2G (mass, momentum, force
 * [, mass gradient]) -> displacement control -> grid update with boundary
 * conditions and friction -> G2P pass 1 -> velocity remap -> boundary
 * conditions / displacement control -> G2P pass 2 with the constitutive
 * increment -> platen timeline, on one NVIDIA GB300 (sm_103a).
 *
 * Conventions
 *   - Every call returns an int status: MPM_OK (0) or a negative MPM_ERR_*;
 *     mpm_last_error() gives the message of the last failure on a context.
 *   - The caller owns every host buffer; the context owns all device memory.
 *   - Per-particle vectors are n x k row-major host arrays (the k components
 *     of particle 0 first); the 3x3 deformation gradient is stored in glm's
 *     column-major element order, F[c][r] at offset 3*c + r
 *     (MaterialPoint_BC.h:52).  Node arrays use the reference's node index
 *     ix + iy*nx + iz*nx*ny (GridPoint_Factory.h:18-22), nx = cells_x + 1.
 *   - A context is not thread-safe; all work is ordered on one CUDA stream.
 *   - No CPU fallback: every compute entry point runs CUDA kernels, and
 *     mpm_create fails when no usable device is present.
 */
#ifndef MPM_GB300_H
#define MPM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPM_OK 0
#define MPM_ERR_ARG (-1)     /* invalid argument or size */
#define MPM_ERR_CUDA (-2)    /* a CUDA runtime call failed */
#define MPM_ERR_STATE (-3)   /* call out of order (e.g. advance before upload) */
#define MPM_ERR_DEVICE (-4)  /* a kernel reported a data error (non-finite position, ...) */
#define MPM_ERR_NOMEM (-5)   /* device allocation failed */
#define MPM_ERR_TOO_LARGE (-6) /* size exceeds the fixed capacity of an entry point that does not allocate */

/* Numerical forms. */
#define MPM_FORM_FP64 0 /* plain form: the reference method in FP64 */
#define MPM_FORM_FP32 1 /* chosen form: FP32 transfers and grid, FP64 positions and energies */

/* Material type ids, as Material_BC.h:6-11. Unknown ids use the PerfectlyPlastic law (…MPLocks.cpp:238). */
#define MPM_MAT_ELASTIC 0
#define MPM_MAT_PLASTIC 3
#define MPM_MAT_VONMISESHARDENING 4

/* Particle flag bits (MaterialPoint_BC.h:32-43). */
#define MPM_PF_DC_X 1u     /* b3_DisplacementControl.x */
#define MPM_PF_DC_Y 2u     /* b3_DisplacementControl.y */
#define MPM_PF_DC_Z 4u     /* b3_DisplacementControl.z */
#define MPM_PF_DC_SKIP 8u  /* b_DisplacementControl: skipped by G2P on the contact path */
#define MPM_PF_SURFACE 16u /* b_Surface: takes part in contact detection */

/* Node fixed bits (GridPoint.h:20, b3_Fixed) and node state bits. */
#define MPM_NF_FIX_X 1u
#define MPM_NF_FIX_Y 2u
#define MPM_NF_FIX_Z 4u
#define MPM_NS_ACTIVE 1u   /* b_Active */
#define MPM_NS_CONTACT 2u  /* b_Contact */
#define MPM_NS_POSITIVE 4u /* b_Contact_Positive */
#define MPM_NS_NEGATIVE 8u /* b_Contact_Negative */

/* Options for mpm_set_option. */
#define MPM_OPT_FLOOR_FRICTION 1 /* contact path: Coulomb friction on x/y of z-fixed nodes (extension; default 0) */
#define MPM_OPT_PROFILE 2        /* 1: time every kernel with CUDA events (default 0) */
#define MPM_OPT_P2G_REDUCE 3     /* P2G: 0 = one atomic per particle, 1 = sum each cell's run across lanes first, 2 = stage the block in shared memory and sum each (cell, corner) in one thread, 3 (default) / 4 = as 2 with each thread summing 2 / 4 corners of a cell */
#define MPM_OPT_P2G_BLOCK 4      /* P2G threads per block (128, 256 or 512) */
#define MPM_OPT_PASS_BLOCK 5     /* G2P pass-2 threads per block (128, 256 (default) or 512) */
#define MPM_OPT_GATHER 6         /* pass-2 (G2P) mode: 0 = node gathers one corner at a time, 1 = several corners'
                                    loads issued together, 2 = (FP32 form) as 0 with the block's particle fields
                                    brought into shared memory by bulk copies first */
#define MPM_OPT_GRAPH 7          /* 1 (default): mpm_advance replays a captured two-step CUDA graph in the steady state; 0: launch every kernel */
#define MPM_OPT_REORDER 8        /* FP32 form: store particles in cell order after each particle upload (0, default), also every N steps (N > 0), or never (-1); results stay in the caller's order */
#define MPM_OPT_PASS1_CORNERS 10 /* cell-run G2P pass 1 (P2G modes 2-4): corners per thread, 1, 2 (default) or 4 */
#define MPM_OPT_PASS1_BLOCK 11   /* cell-run G2P pass 1: threads per block (128, 256 or 512) */
#define MPM_OPT_LARGE_STRAIN 12  /* FP64 form, non-contact loop: 1 runs the large-strain pass 2 (G2P_P2_LargeStrain, PhysicsEngine_runSimulation_Classic_DoublePass_MPLocks.cpp:281-437), which the reference ships disabled (:605); 0 (default) the small-strain pass */
#define MPM_OPT_FP64_FALLBACK 13 /* FP32 form: 1 (default) computes the von Mises hardening return map
                                    (…_VonMisesHardening.cpp:4-92) in FP64 for particles whose FP32 trial yield
                                    function is above -0.001 x k0 and that the network does not take: with a
                                    network the states up to its band (mpm_attach_surrogate, 0.02 by default) past
                                    the surface, every plastic state without one, and the elastic states just
                                    below the surface; 0: FP32 throughout */
#define MPM_OPT_SURROGATE_GUARD 14 /* FP32 form with the learned return map: tolerance of the guard on the network's
                                      results as a fraction of k0 (default 0.001; 0 turns the guard off), see
                                      mpm_attach_surrogate */
#define MPM_OPT_CELL_SORT 9      /* FP32 form, P2G modes 2-4: 1 sorts the particles by cell every step; 0 (default) takes the storage order as it is (a cell whose particles are not adjacent is summed in several runs) and, with MPM_OPT_REORDER 0, restores the cell order every 256 steps */

typedef struct mpm_ctx mpm_ctx;

/* Regular grid: cells[a] cells of size length[a]/cells[a] along axis a
 * (GridPoint_Factory.h:33-68; GridPoint_Mediator.h:25-28). */
typedef struct mpm_grid_desc {
    double length[3];
    int32_t cells[3];
    int32_t pad;
} mpm_grid_desc;

/* Material_BC.h:13-35. */
typedef struct mpm_material {
    int32_t type;
    int32_t pad;
    double density, E, nu, yield, C0, C1;
} mpm_material;

/* Scalars of the time loop (PhysicsEngine.h:83-116). */
typedef struct mpm_sim {
    double time;     /* d_Time */
    double dt_max;   /* d_TimeIncrement_Maximum */
    double mass_min; /* d_Mass_Minimum */
    double damping;  /* d_DampingCoefficient */
    double time_end; /* d_TimeEnd */
    int64_t step;    /* i_TimeCycle */
} mpm_sim;

/* Host views of the particle state (MaterialPoint_BC.h:25-85).  On upload a
 * NULL field takes its default (zero; F = identity; dc_mult = 1); on
 * download a NULL field is skipped. */
typedef struct mpm_particles {
    double *pos, *vel, *fext;        /* n x 3 */
    double *mass, *vol, *vol0;       /* n */
    double* F;                       /* n x 9, column-major */
    double *stress, *strain, *eps_p; /* n x 6, Voigt xx yy zz xy yz zx, engineering shear strain */
    double *e_strain, *e_strain_max, *e_strain_ti, *e_plastic, *backstress; /* n */
    double* mp_mass_gradient;        /* n x 3 (contact path output) */
    double* strain_rate;             /* n x 6 (contact path output) */
    int32_t* material;               /* n, index into the uploaded material table (<0: none) */
    uint8_t* pflags;                 /* n, MPM_PF_* */
    float* dc_mult;                  /* n, f_DisplacementControl_Multiplier */
    int32_t* specimen;               /* n, specimen of each particle (batches only; upload only) */
    double* F_elastic;               /* n x 9, column-major: d33_DeformationGradient_Elastic (MaterialPoint_BC.h:65),
                                        the large-strain pass 2's state; FP64 form (identity when NULL; the FP32
                                        form downloads the identity) */
} mpm_particles;

/* Host views of the node state (GridPoint.h:6-45), n_nodes entries each. */
typedef struct mpm_nodes {
    uint8_t* fixed;        /* MPM_NF_* */
    double* friction;      /* d_FrictionCoefficient */
    double* mass;          /* d_Mass */
    double *mom, *vel, *force, *force_temp, *mass_gradient; /* n_nodes x 3 */
    uint8_t* state;        /* MPM_NS_* */
} mpm_nodes;

/* Per-kernel timing record (MPM_OPT_PROFILE). */
typedef struct mpm_kernel_stat {
    char name[32];
    int64_t launches;
    double total_ms;
} mpm_kernel_stat;

/* --- lifetime --------------------------------------------------------------
 * Replaces the engine set-up the reference scene builders do
 * (GridPoint_Factory::createGrid, GridPoint_Factory.h:33-68, and the mediator
 * geometry, e.g. PhysicsEngine_initializeWorld_Classic_Bar.cpp:15-27). */
int mpm_create(const mpm_grid_desc* grid, int form, mpm_ctx** out);
/* A batch of independent specimens, each with its own grid, advanced together
 * by every launch (no counterpart in the reference, which runs one scene per
 * engine).  Their nodes are numbered one specimen after the other (node
 * arrays in mpm_upload_nodes / mpm_download_nodes are the concatenation);
 * each particle names its specimen (mpm_particles.specimen).  Specimens never
 * share nodes, so each evolves exactly as it would alone. */
int mpm_create_batch(const mpm_grid_desc* grids, int32_t nspec, int form, mpm_ctx** out);
/* node_offsets[0..nspec]: first node of each specimen, then the total. */
int mpm_batch_info(const mpm_ctx* ctx, int64_t* node_offsets, int32_t* nspec);
void mpm_destroy(mpm_ctx* ctx); /* PhysicsEngine::~PhysicsEngine, PhysicsEngine.cpp:4-38 */
const char* mpm_last_error(const mpm_ctx* ctx);
int mpm_device_info(char* name, int name_len, int* sm_count, int* cc_major, int* cc_minor);

/* Use the caller's CUDA stream (cudaStream_t passed as void*) instead of the context's own. */
int mpm_set_stream(mpm_ctx* ctx, void* stream);
int mpm_set_option(mpm_ctx* ctx, int key, double value);

/* --- state transfer ---------------------------------------------------------
 * The reference keeps this state in PhysicsEngine's vectors v_allMaterial,
 * allMaterialPoint, v_MarkedMaterialPoints_Displacement_Control and
 * allGridPoint (PhysicsEngine.h:89-93) and m_TimeLine (:82). */
int mpm_upload_materials(mpm_ctx* ctx, const mpm_material* mats, int32_t n);
int mpm_upload_particles(mpm_ctx* ctx, const mpm_particles* p, int64_t n);
/* Indices of displacement-controlled particles, in the order of
 * v_MarkedMaterialPoints_Displacement_Control (that order decides which
 * particle's velocity a shared node keeps).  Duplicates are rejected. */
int mpm_upload_dc_list(mpm_ctx* ctx, const uint32_t* idx, int64_t n);
int mpm_upload_nodes(mpm_ctx* ctx, const mpm_nodes* nodes);
int mpm_set_timeline(mpm_ctx* ctx, const double* t, const double* v3, int32_t n); /* TimeLine::addTimePoint */
int mpm_set_sim(mpm_ctx* ctx, const mpm_sim* sim);
int mpm_get_sim(const mpm_ctx* ctx, mpm_sim* sim);
int mpm_download_particles(mpm_ctx* ctx, mpm_particles* p);
int mpm_download_nodes(mpm_ctx* ctx, mpm_nodes* nodes);

/* --- time stepping -----------------------------------------------------------
 * mpm_advance: `nsteps` steps of increment dt each, on the context's stream
 * (asynchronous).  contact = 0 is the step of
 * runSimulation_Classic_DoublePass_MPLocks (…MPLocks.cpp:462-792), contact = 1
 * the step of runSimulation_Classic_DoublePass_MPLocks_Contact
 * (…_Contact.cpp:27-543).  Time and step count advance as d_Time += dt,
 * i_TimeCycle++ (…MPLocks.cpp:802-803). */
int mpm_advance(mpm_ctx* ctx, int32_t nsteps, double dt, int contact);
/* mpm_run: the whole while-loop of runSimulation_…(dTimeIncrement_Total)
 * (…MPLocks.cpp:449-458, 806-814) without the console report: steps of
 * dt_max, the last one shortened to end exactly at dt_total; *done = 1 when
 * time >= time_end.  Returns after the work is complete. */
int mpm_run(mpm_ctx* ctx, double dt_total, int contact, int* done);
/* Wait for the stream and surface any device-side error. */
int mpm_synchronize(mpm_ctx* ctx);
/* mpm_advance bracketed by CUDA events on the context's stream; *ms = device time. */
int mpm_advance_timed(mpm_ctx* ctx, int32_t nsteps, double dt, int contact, float* ms);

/* Autotuner (no counterpart in the reference, which has one fixed OpenMP
 * loop): times `steps` steps of dt per candidate launch configuration on the
 * current state in three stages, each keeping the fastest so far: P2G mode x
 * P2G block (15), then pass-1 corners per thread x pass-1 block (9, cell-run
 * modes only), then pass-2 block x pass-2 mode (6; 9 in the FP32 form).  The particle and node
 * state and the time are restored exactly as they were.  Results are the
 * chosen options and the best and worst candidate times per step. */
typedef struct mpm_tune_result {
    int32_t p2g_reduce, p2g_block, pass_block, candidates;
    double best_ms_per_step, worst_ms_per_step;
    int32_t gather_batch, pass1_corners, pass1_block;
} mpm_tune_result;
int mpm_autotune(mpm_ctx* ctx, int32_t steps, double dt, int contact, mpm_tune_result* out);

/* Diagnostics: the cell key of every particle (base cell (bx,by,bz) =
 * floor(x/h) as in GridPoint_Mediator.cpp:8, key = (bx+1) + (cx+2)*((by+1) +
 * (cy+2)*(bz+1)), or (cx+2)(cy+2)(cz+2) when no node is in range) and the
 * particle order sorted by key (stable) used by the last step.  Either
 * pointer may be NULL; n must equal the particle count. */
int mpm_cell_order(mpm_ctx* ctx, uint32_t* keys, uint32_t* sorted_order, int64_t n);

/* --- cell order without allocation --------------------------------------------
 * No counterpart in the reference (which has no device and no allocator to
 * avoid).  For callers that cannot allocate device memory when they need the
 * cell order: code running inside a memory pool or arena that owns the whole
 * device heap, plug-ins whose host framework forbids cudaMalloc/cudaFree on
 * the calling thread, and loops where an allocation (or the device-wide
 * synchronisation of cudaFree) is not acceptable.
 *
 * Computes, for n particles at device positions d_pos (structure of arrays:
 * x[0..n), y[0..n), z[0..n), doubles), the cell key of every particle into
 * d_keys and the particle order sorted stably by key into d_order (both
 * device arrays of n uint32), exactly as mpm_cell_order() reports them.
 * No memory is allocated, by this call or by any routine it calls: the
 * working memory is one fixed array of static device storage inside the
 * library (about 16.3 MiB, sized for MPM_NOALLOC_MAX_PARTICLES), which every
 * GPU that loads the library holds until the process exits.
 *   - n > MPM_NOALLOC_MAX_PARTICLES returns MPM_ERR_TOO_LARGE and does nothing.
 *   - Work is queued on `stream` (a cudaStream_t, NULL for the default
 *     stream); the outputs are ready once that stream has been synchronised.
 *   - All calls share the one scratch array (each call starts by clearing
 *     what it needs), so calls whose work overlaps on the GPU -- on different
 *     streams, or from different threads -- race and corrupt each other's
 *     results: serialise them.
 *   - The first call on each device looks up the scratch array's device
 *     address (a one-time set-up, done with that device current); make that
 *     first call before any stream capture on the device.
 *   - A non-finite position gets the out-of-grid key (the largest key). */
#define MPM_NOALLOC_MAX_PARTICLES (1 << 20)
int mpm_cell_order_noalloc(const mpm_grid_desc* grid, const double* d_pos, int64_t n, uint32_t* d_keys,
                           uint32_t* d_order, void* stream);

/* --- console monitors ---------------------------------------------------------
 * The quantities PhysicsEngine::reportConsole (PhysicsEngine.cpp:40-183)
 * reduces over its marked particle lists, computed on the GPU in FP64 so a
 * host need not download the particles at every console interval.  Particle
 * membership in the reference's lists is given by a per-particle mask. */
#define MPM_MON_DISPLACEMENT 1u /* v_MarkedMaterialPoints_Displacement_Monitor */
#define MPM_MON_MOMENTUM 2u     /* v_MarkedMaterialPoints_Momentum */
#define MPM_MON_PRINCIPAL 4u    /* v_MarkedMaterialPoints_Principal_Monitor */
#define MPM_MON_STRESS 8u       /* v_MarkedMaterialPoints_Stress_Monitor */
#define MPM_MON_ENERGY 16u      /* v_MarkedMaterialPoints_Monitor_Energy */
typedef struct mpm_monitors {
    double time;
    double position_mean[3];  /* displacement list: mean position (:48-59) */
    double force_sum[3];      /* all nodes: sum of d3_Force_Temp (:61-70) */
    double momentum[3];       /* momentum list: sum of m v (:72-80) */
    double strain_p_max;      /* principal list: max |principal strain| (:82-120) */
    double stress_p_max;      /* principal list: max |principal stress| */
    double stress_mean[3];    /* stress list: mean sigma_xx, sigma_yy, sigma_zz (:122-138) */
    double strain_mean[3];    /* stress list: mean eps_xx, eps_yy, eps_zz */
    double kinetic;           /* energy list: sum 0.5 m |v|^2 (:140-156) */
    double strain_energy;     /* energy list: sum of d_Energy_Strain */
    double plastic_energy;    /* energy list: sum of d_Energy_Plastic */
    int64_t count[5];         /* members of each list, in the order of the MPM_MON_* bits */
    /* Boundary work since the last mpm_upload_particles, accumulated in FP64
     * every step (no counterpart in the reference, whose report has no
     * external-work term).  platen_work: the work of displacement control,
     * sum over controlled node axes of -f v dt (f: the node's force the
     * control zeroes, v: the velocity it imposes, …MPLocks.cpp:143-174,
     * …_Contact.cpp:283-297).  friction_work: the work of the friction laws,
     * sum of df (p/m) dt (df: the force a friction law adds to a tangent,
     * p/m: the node's updated velocity; dissipation, so <= 0).  The strain
     * energy is the stress work, plastic dissipation included, so
     * kinetic + strain_energy - (initial values) - platen_work - friction_work
     * is the discrete energy balance's residual. */
    double platen_work;
    double friction_work;
} mpm_monitors;
int mpm_upload_monitor_mask(mpm_ctx* ctx, const uint8_t* mask, int64_t n);
int mpm_monitors_read(mpm_ctx* ctx, mpm_monitors* out);

/* --- profiling ---------------------------------------------------------------
 * Per-kernel CUDA-event timers (the reference's a_Runtime, PhysicsEngine.h:87). */
int mpm_profile_read(mpm_ctx* ctx, mpm_kernel_stat* out, int32_t max, int32_t* count);
int mpm_profile_reset(mpm_ctx* ctx);
/* Number of kernels the engine launched since creation (all kinds). */
int mpm_launch_count(const mpm_ctx* ctx, int64_t* count);

#ifdef __cplusplus
}
#endif

#endif /* MPM_GB300_H */
