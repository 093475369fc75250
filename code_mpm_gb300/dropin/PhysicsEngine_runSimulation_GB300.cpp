// Drop-in replacement for
//   PhysicsEngine_runSimulation_Classic_DoublePass_MPLocks.cpp
//   PhysicsEngine_runSimulation_Classic_DoublePass_MPLocks_Contact.cpp
// of code_MPM: link this file (and libmpm_gb300.so) instead of those two, and
// PhysicsEngine::runSimulation_Classic_DoublePass_MPLocks(double) and
// ::runSimulation_Classic_DoublePass_MPLocks_Contact(double) (PhysicsEngine.h:54-55)
// run on the GPU through the C ABI of include/mpm_gb300.h.
//
// Each call packs the engine's heap objects (allMaterialPoint, allGridPoint,
// v_allMaterial, v_MarkedMaterialPoints_Displacement_Control, m_TimeLine)
// into the structure-of-arrays views, advances step by step with the
// reference's time chunking (…MPLocks.cpp:449-458), reports to the console at
// the reference's interval (:796-800) after pulling the state back, and on
// return leaves every MaterialPoint_BC / GridPoint field current, so callers
// that read or edit the objects between calls (the viewer, the ESO loop) see
// what the CPU solver would have left.
//
// The GPU state is set up anew on every call: the host objects are the state
// of record, as they are for the reference.
#include <cstdio>
#include <map>
#include <vector>

#include "PhysicsEngine.h"
#include "mpm_gb300.h"

namespace {

struct Packed {
    std::vector<double> pos, vel, fext, mass, vol, vol0, F, Fe, stress, strain, eps_p, e_s, e_smax, e_sti, e_p, R, mg,
        rate;
    std::vector<int32_t> material;
    std::vector<uint8_t> flags;
    std::vector<float> mult;
    void resize(size_t n) {
        pos.resize(3 * n); vel.resize(3 * n); fext.resize(3 * n); mass.resize(n); vol.resize(n); vol0.resize(n);
        F.resize(9 * n); Fe.resize(9 * n); stress.resize(6 * n); strain.resize(6 * n); eps_p.resize(6 * n); e_s.resize(n);
        e_smax.resize(n); e_sti.resize(n); e_p.resize(n); R.resize(n); mg.resize(3 * n); rate.resize(6 * n);
        material.resize(n); flags.resize(n); mult.resize(n);
    }
    mpm_particles view() {
        mpm_particles v = {};
        v.pos = pos.data(); v.vel = vel.data(); v.fext = fext.data(); v.mass = mass.data(); v.vol = vol.data();
        v.vol0 = vol0.data(); v.F = F.data(); v.stress = stress.data(); v.strain = strain.data();
        v.eps_p = eps_p.data(); v.e_strain = e_s.data(); v.e_strain_max = e_smax.data(); v.e_strain_ti = e_sti.data();
        v.e_plastic = e_p.data(); v.backstress = R.data(); v.mp_mass_gradient = mg.data(); v.strain_rate = rate.data();
        v.material = material.data(); v.pflags = flags.data(); v.dc_mult = mult.data(); v.F_elastic = Fe.data();
        return v;
    }
};

struct PackedNodes {
    std::vector<uint8_t> fixed, state;
    std::vector<double> friction, mass, mom, vel, force, ftemp, mg;
    void resize(size_t n) {
        fixed.resize(n); state.resize(n); friction.resize(n); mass.resize(n); mom.resize(3 * n); vel.resize(3 * n);
        force.resize(3 * n); ftemp.resize(3 * n); mg.resize(3 * n);
    }
    mpm_nodes view() {
        mpm_nodes v = {};
        v.fixed = fixed.data(); v.friction = friction.data(); v.mass = mass.data(); v.mom = mom.data();
        v.vel = vel.data(); v.force = force.data(); v.force_temp = ftemp.data(); v.mass_gradient = mg.data();
        v.state = state.data();
        return v;
    }
};

void pack_particle(const MaterialPoint_BC* mp, size_t p, const std::map<const Material_BC*, int>& mats, Packed& P) {
    for (int k = 0; k < 3; ++k) {
        P.pos[3 * p + k] = mp->d3_Position[k];
        P.vel[3 * p + k] = mp->d3_Velocity[k];
        P.fext[3 * p + k] = mp->d3_Force_External[k];
        P.mg[3 * p + k] = mp->d3_MassGradient[k];
    }
    P.mass[p] = mp->d_Mass;
    P.vol[p] = mp->d_Volume;
    P.vol0[p] = mp->d_Volume_Initial;
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) {
            P.F[9 * p + 3 * c + r] = mp->d33_DeformationGradient[c][r];
            P.Fe[9 * p + 3 * c + r] = mp->d33_DeformationGradient_Elastic[c][r];
        }
    for (int k = 0; k < 6; ++k) {
        P.stress[6 * p + k] = mp->d6_Stress[k];
        P.strain[6 * p + k] = mp->d6_Strain[k];
        P.eps_p[6 * p + k] = mp->d6_Strain_Plastic[k];
        P.rate[6 * p + k] = mp->d6_Strain_Rate[k];
    }
    P.e_s[p] = mp->d_Energy_Strain;
    P.e_smax[p] = mp->d_Energy_Strain_MaxHistory;
    P.e_sti[p] = mp->d_Energy_Strain_TimeIntegral;
    P.e_p[p] = mp->d_Energy_Plastic;
    P.R[p] = mp->d_BackStress_Isotropic;
    auto it = mats.find(mp->p_Material);
    P.material[p] = it == mats.end() ? -1 : it->second;
    P.flags[p] = (uint8_t)((mp->b3_DisplacementControl.x ? MPM_PF_DC_X : 0) |
                           (mp->b3_DisplacementControl.y ? MPM_PF_DC_Y : 0) |
                           (mp->b3_DisplacementControl.z ? MPM_PF_DC_Z : 0) |
                           (mp->b_DisplacementControl ? MPM_PF_DC_SKIP : 0) | (mp->b_Surface ? MPM_PF_SURFACE : 0));
    P.mult[p] = mp->f_DisplacementControl_Multiplier;
}

void unpack_particle(MaterialPoint_BC* mp, size_t p, const Packed& P) {
    for (int k = 0; k < 3; ++k) {
        mp->d3_Position[k] = P.pos[3 * p + k];
        mp->d3_Velocity[k] = P.vel[3 * p + k];
        mp->d3_MassGradient[k] = P.mg[3 * p + k];
    }
    mp->d_Volume = P.vol[p];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) {
            mp->d33_DeformationGradient[c][r] = P.F[9 * p + 3 * c + r];
            mp->d33_DeformationGradient_Elastic[c][r] = P.Fe[9 * p + 3 * c + r];
        }
    for (int k = 0; k < 6; ++k) {
        mp->d6_Stress[k] = P.stress[6 * p + k];
        mp->d6_Strain[k] = P.strain[6 * p + k];
        mp->d6_Strain_Plastic[k] = P.eps_p[6 * p + k];
        mp->d6_Strain_Rate[k] = P.rate[6 * p + k];
    }
    mp->d_Energy_Strain = P.e_s[p];
    mp->d_Energy_Strain_MaxHistory = P.e_smax[p];
    mp->d_Energy_Strain_TimeIntegral = P.e_sti[p];
    mp->d_Energy_Plastic = P.e_p[p];
    mp->d_BackStress_Isotropic = P.R[p];
}

int fail(mpm_ctx* ctx, int rc) {
    fprintf(stderr, "GB300 MPM engine error %d: %s\n", rc, mpm_last_error(ctx));
    return rc;
}

}  // namespace

// One routine for both solvers; `contact` selects the step.
static int gb300_run(PhysicsEngine* self, double total, int contact, std::vector<MaterialPoint_BC*>& mps,
                     std::vector<GridPoint*>& gps, std::vector<Material_BC*>& materials,
                     std::vector<MaterialPoint_BC*>& dc, TimeLine& timeline, const GridPoint_Mediator& geom,
                     double& time, int& cycle, double dt_max, double mass_min, double damping, double time_end,
                     double& console_last, double console_interval, double& runtime,
                     void (PhysicsEngine::*report)(std::string));

int PhysicsEngine::runSimulation_Classic_DoublePass_MPLocks(double dTimeIncrement_Total) {
    return gb300_run(this, dTimeIncrement_Total, 0, allMaterialPoint, allGridPoint, v_allMaterial,
                     v_MarkedMaterialPoints_Displacement_Control, m_TimeLine, mpm_GP_Mediator_Thread[0], d_Time,
                     i_TimeCycle, d_TimeIncrement_Maximum, d_Mass_Minimum, d_DampingCoefficient, d_TimeEnd,
                     d_TimeConsole_Last, d_TimeConsole_Interval, d_Runtime_Total, &PhysicsEngine::reportConsole);
}

int PhysicsEngine::runSimulation_Classic_DoublePass_MPLocks_Contact(double dTimeIncrement_Total) {
    return gb300_run(this, dTimeIncrement_Total, 1, allMaterialPoint, allGridPoint, v_allMaterial,
                     v_MarkedMaterialPoints_Displacement_Control, m_TimeLine, mpm_GP_Mediator_Thread[0], d_Time,
                     i_TimeCycle, d_TimeIncrement_Maximum, d_Mass_Minimum, d_DampingCoefficient, d_TimeEnd,
                     d_TimeConsole_Last, d_TimeConsole_Interval, d_Runtime_Total, &PhysicsEngine::reportConsole);
}

static int gb300_run(PhysicsEngine* self, double total, int contact, std::vector<MaterialPoint_BC*>& mps,
                     std::vector<GridPoint*>& gps, std::vector<Material_BC*>& materials,
                     std::vector<MaterialPoint_BC*>& dc, TimeLine& timeline, const GridPoint_Mediator& geom,
                     double& time, int& cycle, double dt_max, double mass_min, double damping, double time_end,
                     double& console_last, double console_interval, double& runtime,
                     void (PhysicsEngine::*report)(std::string)) {
    double t_start = omp_get_wtime();
    mpm_grid_desc gd = {};
    for (int a = 0; a < 3; ++a) {
        gd.length[a] = geom.d3_Length_Grid[a];
        gd.cells[a] = geom.i3_Cells[a];
    }
    mpm_ctx* ctx = nullptr;
    int rc = mpm_create(&gd, MPM_FORM_FP64, &ctx);
    if (rc) return fail(ctx, rc);
    // materials (pointer -> table index)
    std::map<const Material_BC*, int> mat_index;
    std::vector<mpm_material> mt(materials.size());
    for (size_t i = 0; i < materials.size(); ++i) {
        mat_index[materials[i]] = (int)i;
        mt[i].type = (int32_t)materials[i]->i_MaterialType;
        mt[i].density = materials[i]->d_Density;
        mt[i].E = materials[i]->d_ElasticModulus;
        mt[i].nu = materials[i]->d_PoissonRatio;
        mt[i].yield = materials[i]->d_YieldStress;
        mt[i].C0 = materials[i]->d_Hardening_Isotropic_C0;
        mt[i].C1 = materials[i]->d_Hardening_Isotropic_C1;
    }
    if ((rc = mpm_upload_materials(ctx, mt.data(), (int32_t)mt.size()))) return fail(ctx, rc);
    // particles
    const size_t n = mps.size();
    Packed P;
    P.resize(n);
    std::map<const MaterialPoint_BC*, uint32_t> mp_index;
    for (size_t p = 0; p < n; ++p) {
        pack_particle(mps[p], p, mat_index, P);
        mp_index[mps[p]] = (uint32_t)p;
    }
    mpm_particles pv = P.view();
    if ((rc = mpm_upload_particles(ctx, &pv, (int64_t)n))) return fail(ctx, rc);
    std::vector<uint32_t> dcl;
    for (MaterialPoint_BC* mp : dc) dcl.push_back(mp_index.at(mp));
    if ((rc = mpm_upload_dc_list(ctx, dcl.data(), (int64_t)dcl.size()))) return fail(ctx, rc);
    // nodes
    const size_t nn = gps.size();
    PackedNodes G;
    G.resize(nn);
    for (size_t i = 0; i < nn; ++i) {
        const GridPoint* gp = gps[i];
        G.fixed[i] = (uint8_t)((gp->b3_Fixed.x ? MPM_NF_FIX_X : 0) | (gp->b3_Fixed.y ? MPM_NF_FIX_Y : 0) |
                               (gp->b3_Fixed.z ? MPM_NF_FIX_Z : 0));
        G.friction[i] = gp->d_FrictionCoefficient;
        G.mass[i] = gp->d_Mass;
        for (int k = 0; k < 3; ++k) {
            G.mom[3 * i + k] = gp->d3_Momentum[k];
            G.vel[3 * i + k] = gp->d3_Velocity[k];
            G.force[3 * i + k] = gp->d3_Force[k];
            G.ftemp[3 * i + k] = gp->d3_Force_Temp[k];
            G.mg[3 * i + k] = gp->d3_MassGradient[k];
        }
        G.state[i] = (uint8_t)((gp->b_Active ? MPM_NS_ACTIVE : 0) | (gp->b_Contact ? MPM_NS_CONTACT : 0) |
                               (gp->b_Contact_Positive ? MPM_NS_POSITIVE : 0) |
                               (gp->b_Contact_Negative ? MPM_NS_NEGATIVE : 0));
    }
    mpm_nodes nv = G.view();
    if ((rc = mpm_upload_nodes(ctx, &nv))) return fail(ctx, rc);
    std::vector<double> tv;
    for (const glm::dvec3& v : timeline.v_Velocity) tv.insert(tv.end(), {v.x, v.y, v.z});
    if ((rc = mpm_set_timeline(ctx, timeline.v_Time.data(), tv.data(), (int32_t)timeline.v_Time.size())))
        return fail(ctx, rc);

    auto pull = [&]() -> int {
        int r = mpm_download_particles(ctx, &pv);
        if (!r) r = mpm_download_nodes(ctx, &nv);
        if (r) return r;
        for (size_t p = 0; p < n; ++p) unpack_particle(mps[p], p, P);
        for (size_t i = 0; i < nn; ++i) {
            GridPoint* gp = gps[i];
            gp->d_Mass = G.mass[i];
            for (int k = 0; k < 3; ++k) {
                gp->d3_Momentum[k] = G.mom[3 * i + k];
                gp->d3_Velocity[k] = G.vel[3 * i + k];
                gp->d3_Force[k] = G.force[3 * i + k];
                gp->d3_Force_Temp[k] = G.ftemp[3 * i + k];
                gp->d3_MassGradient[k] = G.mg[3 * i + k];
            }
            gp->b_Active = (G.state[i] & MPM_NS_ACTIVE) != 0;
            gp->b_Contact = (G.state[i] & MPM_NS_CONTACT) != 0;
            gp->b_Contact_Positive = (G.state[i] & MPM_NS_POSITIVE) != 0;
            gp->b_Contact_Negative = (G.state[i] & MPM_NS_NEGATIVE) != 0;
        }
        return 0;
    };

    // …MPLocks.cpp:449-458 time chunking, :796-803 console and time advance.
    // The steps between two console reports have one size, so each such run
    // goes to the GPU in one mpm_advance call (which replays the step graph);
    // the host then repeats the reference's bookkeeping for the run.
    mpm_sim sim = {time, dt_max, mass_min, damping, time_end, (int64_t)cycle};
    if ((rc = mpm_set_sim(ctx, &sim))) return fail(ctx, rc);
    double acc = 0.0;
    while (acc < total) {
        int k = 0;
        double run_dt = 0.0;
        {
            double a = acc, t = time;
            while (a < total) {
                double dt = dt_max;
                if (dt_max > (total - a)) dt = total - a;
                if (k > 0 && dt != run_dt) break;
                run_dt = dt;
                a += dt;
                ++k;
                const bool console = t - console_last > console_interval;
                t += dt;
                if (console) break;
            }
        }
        if ((rc = mpm_advance(ctx, k, run_dt, contact))) return fail(ctx, rc);
        for (int i = 0; i < k; ++i) {
            acc += run_dt;
            if (time - console_last > console_interval) {  // only the run's last step can report
                if ((rc = pull())) return fail(ctx, rc);
                console_last = time;
                (self->*report)("");
            }
            time += run_dt;
            cycle++;
        }
    }
    if ((rc = mpm_synchronize(ctx)) || (rc = pull())) return fail(ctx, rc);
    mpm_destroy(ctx);
    runtime += omp_get_wtime() - t_start;
    if (time < time_end) return 0;
    console_last = time;
    (self->*report)("");
    std::cout << "Analysis complete ..." << std::endl;
    return 1;
}
