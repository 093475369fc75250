// mpm_dropin.hpp -- a resident engine session over code_MPM's own solver objects.
//
// The drop-in translation unit (PhysicsEngine_runSimulation_GB300.cpp) replaces
// PhysicsEngine::runSimulation_Classic_DoublePass_MPLocks(double) and
// ::runSimulation_Classic_DoublePass_MPLocks_Contact(double) (PhysicsEngine.h:54-55).
// This header holds everything of it that does not name PhysicsEngine:
//   - the field mapping between the reference's objects (MaterialPoint_BC.h:25-85,
//     GridPoint.h:6-45, Material_BC.h:13-35, TimeLine.h) and the structure-of-arrays
//     views of the C ABI (include/mpm_gb300.h);
//   - Session, which keeps one engine context resident across calls: it packs
//     and uploads the objects on first use, and again only when the particle
//     list is not the one it left (another count, another object at some
//     index, or an object whose position differs from what the session wrote
//     into it), or after invalidate();
//   - Session::run, the reference's time loop (…MPLocks.cpp:449-458 chunking,
//     :796-814 console report and return value) around mpm_advance.
// It is templated on the object types, so it compiles against the reference's
// classes and against any types with the same member names.
//
// The objects stay the state of record for the caller: at every console
// report and at the end of every run the device state is copied back into
// every particle and node object.  Between runs the device holds the same
// state; a caller that edits fields other than positions between runs (a
// particle's stress, a node's boundary flags, ...) calls invalidate() so the
// next run re-packs.
#pragma once

#include <cstdint>
#include <cstdio>
#include <map>
#include <type_traits>
#include <utility>
#include <vector>

#include "mpm_gb300.h"

namespace mpm_dropin {

// Members the reference's own headers comment out (MaterialPoint_BC.h:33,51,71;
// GridPoint.h:26) while its contact loop uses them: mapped where the type has them.
template <class T, class = void>
struct has_dc_skip : std::false_type {};
template <class T>
struct has_dc_skip<T, std::void_t<decltype(std::declval<T&>().b_DisplacementControl)>> : std::true_type {};
template <class T, class = void>
struct has_mass_gradient : std::false_type {};
template <class T>
struct has_mass_gradient<T, std::void_t<decltype(std::declval<T&>().d3_MassGradient)>> : std::true_type {};
template <class T, class = void>
struct has_strain_rate : std::false_type {};
template <class T>
struct has_strain_rate<T, std::void_t<decltype(std::declval<T&>().d6_Strain_Rate)>> : std::true_type {};

// Host structure-of-arrays copy of the particle state (n x k row-major, as the ABI takes it).
struct ParticleArrays {
    std::vector<double> pos, vel, fext, mass, vol, vol0, F, Fe, stress, strain, eps_p, e_s, e_smax, e_sti, e_p, R, mg,
        rate;
    std::vector<int32_t> material;
    std::vector<uint8_t> flags;
    std::vector<float> mult;
    void resize(size_t n) {
        for (auto* v : {&pos, &vel, &fext, &mg}) v->assign(3 * n, 0.0);
        for (auto* v : {&mass, &vol, &vol0, &e_s, &e_smax, &e_sti, &e_p, &R}) v->assign(n, 0.0);
        for (auto* v : {&F, &Fe}) v->assign(9 * n, 0.0);
        for (auto* v : {&stress, &strain, &eps_p, &rate}) v->assign(6 * n, 0.0);
        material.assign(n, -1);
        flags.assign(n, 0);
        mult.assign(n, 1.0f);
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

struct NodeArrays {
    std::vector<uint8_t> fixed, state;
    std::vector<double> friction, mass, mom, vel, force, ftemp, mg;
    void resize(size_t n) {
        fixed.assign(n, 0);
        state.assign(n, 0);
        friction.assign(n, 0.0);
        mass.assign(n, 0.0);
        for (auto* v : {&mom, &vel, &force, &ftemp, &mg}) v->assign(3 * n, 0.0);
    }
    mpm_nodes view() {
        mpm_nodes v = {};
        v.fixed = fixed.data(); v.friction = friction.data(); v.mass = mass.data(); v.mom = mom.data();
        v.vel = vel.data(); v.force = force.data(); v.force_temp = ftemp.data(); v.mass_gradient = mg.data();
        v.state = state.data();
        return v;
    }
};

// MaterialPoint_BC -> arrays.  mat: material object -> index in the uploaded table.
template <class MP>
void pack_particle(const MP& mp, size_t p, const std::map<const void*, int>& mat, ParticleArrays& P) {
    for (int k = 0; k < 3; ++k) {
        P.pos[3 * p + k] = mp.d3_Position[k];
        P.vel[3 * p + k] = mp.d3_Velocity[k];
        P.fext[3 * p + k] = mp.d3_Force_External[k];
        if constexpr (has_mass_gradient<MP>::value) P.mg[3 * p + k] = mp.d3_MassGradient[k];
    }
    P.mass[p] = mp.d_Mass;
    P.vol[p] = mp.d_Volume;
    P.vol0[p] = mp.d_Volume_Initial;
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) {  // glm column-major: [c][r]
            P.F[9 * p + 3 * c + r] = mp.d33_DeformationGradient[c][r];
            P.Fe[9 * p + 3 * c + r] = mp.d33_DeformationGradient_Elastic[c][r];
        }
    for (int k = 0; k < 6; ++k) {
        P.stress[6 * p + k] = mp.d6_Stress[k];
        P.strain[6 * p + k] = mp.d6_Strain[k];
        P.eps_p[6 * p + k] = mp.d6_Strain_Plastic[k];
        if constexpr (has_strain_rate<MP>::value) P.rate[6 * p + k] = mp.d6_Strain_Rate[k];
    }
    P.e_s[p] = mp.d_Energy_Strain;
    P.e_smax[p] = mp.d_Energy_Strain_MaxHistory;
    P.e_sti[p] = mp.d_Energy_Strain_TimeIntegral;
    P.e_p[p] = mp.d_Energy_Plastic;
    P.R[p] = mp.d_BackStress_Isotropic;
    auto it = mat.find((const void*)mp.p_Material);
    P.material[p] = it == mat.end() ? -1 : it->second;
    uint8_t fl = (uint8_t)((mp.b3_DisplacementControl.x ? MPM_PF_DC_X : 0u) |
                           (mp.b3_DisplacementControl.y ? MPM_PF_DC_Y : 0u) |
                           (mp.b3_DisplacementControl.z ? MPM_PF_DC_Z : 0u) | (mp.b_Surface ? MPM_PF_SURFACE : 0u));
    if constexpr (has_dc_skip<MP>::value) fl |= mp.b_DisplacementControl ? MPM_PF_DC_SKIP : 0u;
    P.flags[p] = fl;
    P.mult[p] = mp.f_DisplacementControl_Multiplier;
}

// arrays -> MaterialPoint_BC: the fields a step writes.
template <class MP>
void unpack_particle(MP& mp, size_t p, const ParticleArrays& P) {
    for (int k = 0; k < 3; ++k) {
        mp.d3_Position[k] = P.pos[3 * p + k];
        mp.d3_Velocity[k] = P.vel[3 * p + k];
        if constexpr (has_mass_gradient<MP>::value) mp.d3_MassGradient[k] = P.mg[3 * p + k];
    }
    mp.d_Volume = P.vol[p];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) {
            mp.d33_DeformationGradient[c][r] = P.F[9 * p + 3 * c + r];
            mp.d33_DeformationGradient_Elastic[c][r] = P.Fe[9 * p + 3 * c + r];
        }
    for (int k = 0; k < 6; ++k) {
        mp.d6_Stress[k] = P.stress[6 * p + k];
        mp.d6_Strain[k] = P.strain[6 * p + k];
        mp.d6_Strain_Plastic[k] = P.eps_p[6 * p + k];
        if constexpr (has_strain_rate<MP>::value) mp.d6_Strain_Rate[k] = P.rate[6 * p + k];
    }
    mp.d_Energy_Strain = P.e_s[p];
    mp.d_Energy_Strain_MaxHistory = P.e_smax[p];
    mp.d_Energy_Strain_TimeIntegral = P.e_sti[p];
    mp.d_Energy_Plastic = P.e_p[p];
    mp.d_BackStress_Isotropic = P.R[p];
}

template <class GP>
void pack_node(const GP& gp, size_t i, NodeArrays& G) {
    G.fixed[i] = (uint8_t)((gp.b3_Fixed.x ? MPM_NF_FIX_X : 0u) | (gp.b3_Fixed.y ? MPM_NF_FIX_Y : 0u) |
                           (gp.b3_Fixed.z ? MPM_NF_FIX_Z : 0u));
    G.friction[i] = gp.d_FrictionCoefficient;
    G.mass[i] = gp.d_Mass;
    for (int k = 0; k < 3; ++k) {
        G.mom[3 * i + k] = gp.d3_Momentum[k];
        G.vel[3 * i + k] = gp.d3_Velocity[k];
        G.force[3 * i + k] = gp.d3_Force[k];
        G.ftemp[3 * i + k] = gp.d3_Force_Temp[k];
        if constexpr (has_mass_gradient<GP>::value) G.mg[3 * i + k] = gp.d3_MassGradient[k];
    }
    G.state[i] = (uint8_t)((gp.b_Active ? MPM_NS_ACTIVE : 0u) | (gp.b_Contact ? MPM_NS_CONTACT : 0u) |
                           (gp.b_Contact_Positive ? MPM_NS_POSITIVE : 0u) |
                           (gp.b_Contact_Negative ? MPM_NS_NEGATIVE : 0u));
}

template <class GP>
void unpack_node(GP& gp, size_t i, const NodeArrays& G) {
    gp.d_Mass = G.mass[i];
    for (int k = 0; k < 3; ++k) {
        gp.d3_Momentum[k] = G.mom[3 * i + k];
        gp.d3_Velocity[k] = G.vel[3 * i + k];
        gp.d3_Force[k] = G.force[3 * i + k];
        gp.d3_Force_Temp[k] = G.ftemp[3 * i + k];
        if constexpr (has_mass_gradient<GP>::value) gp.d3_MassGradient[k] = G.mg[3 * i + k];
    }
    gp.b_Active = (G.state[i] & MPM_NS_ACTIVE) != 0;
    gp.b_Contact = (G.state[i] & MPM_NS_CONTACT) != 0;
    gp.b_Contact_Positive = (G.state[i] & MPM_NS_POSITIVE) != 0;
    gp.b_Contact_Negative = (G.state[i] & MPM_NS_NEGATIVE) != 0;
}

template <class MAT>
mpm_material pack_material(const MAT& m) {
    mpm_material t = {};
    t.type = (int32_t)m.i_MaterialType;
    t.density = m.d_Density;
    t.E = m.d_ElasticModulus;
    t.nu = m.d_PoissonRatio;
    t.yield = m.d_YieldStress;
    t.C0 = m.d_Hardening_Isotropic_C0;
    t.C1 = m.d_Hardening_Isotropic_C1;
    return t;
}

// The scalars of the reference's time loop (PhysicsEngine.h:83-116), by reference
// into the caller's own members so the loop updates them as the reference does.
struct Clock {
    double& time;            // d_Time
    int& cycle;              // i_TimeCycle
    double dt_max;           // d_TimeIncrement_Maximum
    double mass_min;         // d_Mass_Minimum
    double damping;          // d_DampingCoefficient
    double time_end;         // d_TimeEnd
    double& console_last;    // d_TimeConsole_Last
    double console_interval; // d_TimeConsole_Interval
};

// One engine context kept across calls for one solver instance.
template <class MP, class GP, class MAT>
class Session {
  public:
    explicit Session(int form = MPM_FORM_FP64) : form_(form) {}
    Session(const Session&) = delete;
    Session& operator=(const Session&) = delete;
    ~Session() { reset(); }

    void reset() {
        if (ctx_) mpm_destroy(ctx_);
        ctx_ = nullptr;
        mps_.clear();
        pos_.clear();
    }
    // The next attach re-packs and re-uploads everything.
    void invalidate() { stale_ = true; }
    mpm_ctx* context() const { return ctx_; }
    long long uploads() const { return uploads_; }
    const char* error() const { return ctx_ ? mpm_last_error(ctx_) : err_; }

    // Make the device state current for these objects (and the loop's scalars).
    int attach(const mpm_grid_desc& grid, const std::vector<MP*>& mps, const std::vector<GP*>& gps,
               const std::vector<MAT*>& mats, const std::vector<MP*>& dc, const std::vector<double>& tl_t,
               const std::vector<double>& tl_v3, const Clock& clk) {
        int rc;
        const bool same_grid = ctx_ && grid.length[0] == grid_.length[0] && grid.length[1] == grid_.length[1] &&
                               grid.length[2] == grid_.length[2] && grid.cells[0] == grid_.cells[0] &&
                               grid.cells[1] == grid_.cells[1] && grid.cells[2] == grid_.cells[2];
        if (!same_grid) {
            reset();
            grid_ = grid;
            if ((rc = mpm_create(&grid, form_, &ctx_))) {
                ctx_ = nullptr;
                err_ = "mpm_create failed (no usable CUDA device, or a bad grid)";
                return rc;
            }
            stale_ = true;
        }
        // materials: pointer -> table index; re-uploaded when the table changes
        std::map<const void*, int> mat_index;
        std::vector<mpm_material> mt(mats.size());
        for (size_t i = 0; i < mats.size(); ++i) {
            mat_index[(const void*)mats[i]] = (int)i;
            mt[i] = pack_material(*mats[i]);
        }
        if (stale_ || !same_materials(mt)) {
            if ((rc = mpm_upload_materials(ctx_, mt.data(), (int32_t)mt.size()))) return rc;
            mats_ = mt;
            stale_ = true;  // indices into the table may have moved
        }
        if (stale_ || !same_particles(mps)) {
            const size_t n = mps.size();
            P_.resize(n);
            std::map<const MP*, uint32_t> mp_index;
            for (size_t p = 0; p < n; ++p) {
                pack_particle(*mps[p], p, mat_index, P_);
                mp_index[mps[p]] = (uint32_t)p;
            }
            mpm_particles pv = P_.view();
            if ((rc = mpm_upload_particles(ctx_, &pv, (int64_t)n))) return rc;
            std::vector<uint32_t> dcl;
            dcl.reserve(dc.size());
            for (MP* mp : dc) {
                auto it = mp_index.find(mp);
                if (it == mp_index.end()) {
                    err_ = "a displacement-controlled particle is not in the particle list";
                    return MPM_ERR_ARG;
                }
                dcl.push_back(it->second);
            }
            if ((rc = mpm_upload_dc_list(ctx_, dcl.data(), (int64_t)dcl.size()))) return rc;
            G_.resize(gps.size());
            for (size_t i = 0; i < gps.size(); ++i) pack_node(*gps[i], i, G_);
            mpm_nodes nv = G_.view();
            if ((rc = mpm_upload_nodes(ctx_, &nv))) return rc;
            remember(mps);
            ++uploads_;
            stale_ = false;
        }
        if (tl_t != tl_t_ || tl_v3 != tl_v_) {
            if ((rc = mpm_set_timeline(ctx_, tl_t.data(), tl_v3.data(), (int32_t)tl_t.size()))) return rc;
            tl_t_ = tl_t;
            tl_v_ = tl_v3;
        }
        mpm_sim sim = {clk.time, clk.dt_max, clk.mass_min, clk.damping, clk.time_end, (int64_t)clk.cycle};
        return mpm_set_sim(ctx_, &sim);
    }

    // Copy the device state into every particle and node object.
    int detach(const std::vector<MP*>& mps, const std::vector<GP*>& gps) {
        int rc;
        mpm_particles pv = P_.view();
        mpm_nodes nv = G_.view();
        if ((rc = mpm_download_particles(ctx_, &pv)) || (rc = mpm_download_nodes(ctx_, &nv))) return rc;
        for (size_t p = 0; p < mps.size(); ++p) unpack_particle(*mps[p], p, P_);
        for (size_t i = 0; i < gps.size(); ++i) unpack_node(*gps[i], i, G_);
        remember(mps);
        return MPM_OK;
    }

    // runSimulation_…(dTimeIncrement_Total): steps of dt_max, the last one
    // shortened to end at the total (…MPLocks.cpp:449-458); a console report
    // wherever the reference reports (:796-800), with the objects brought up
    // to date first; time and cycle advanced as the reference does
    // (:802-803); 1 once time >= time_end, after a final report (:806-814),
    // else 0.  The steps between two reports have one size, so each such run
    // goes to the GPU in one mpm_advance call.  Negative: an engine error.
    template <class Report>
    int run(double total, int contact, Clock& clk, const std::vector<MP*>& mps, const std::vector<GP*>& gps,
            Report&& report) {
        int rc;
        double acc = 0.0;
        while (acc < total) {
            int k = 0;
            double run_dt = 0.0;
            {
                double a = acc, t = clk.time;
                while (a < total) {
                    double dt = clk.dt_max;
                    if (clk.dt_max > (total - a)) dt = total - a;
                    if (k > 0 && dt != run_dt) break;
                    run_dt = dt;
                    a += dt;
                    ++k;
                    const bool console = t - clk.console_last > clk.console_interval;
                    t += dt;
                    if (console) break;
                }
            }
            if ((rc = mpm_advance(ctx_, k, run_dt, contact))) return rc;
            for (int i = 0; i < k; ++i) {
                acc += run_dt;
                if (clk.time - clk.console_last > clk.console_interval) {  // only the run's last step can report
                    if ((rc = detach(mps, gps))) return rc;
                    clk.console_last = clk.time;
                    report();
                }
                clk.time += run_dt;
                clk.cycle++;
            }
        }
        if ((rc = mpm_synchronize(ctx_)) || (rc = detach(mps, gps))) return rc;
        if (clk.time < clk.time_end) return 0;
        clk.console_last = clk.time;
        report();
        return 1;
    }

  private:
    bool same_materials(const std::vector<mpm_material>& mt) const {
        if (mt.size() != mats_.size()) return false;
        for (size_t i = 0; i < mt.size(); ++i) {
            const mpm_material &a = mt[i], &b = mats_[i];
            if (a.type != b.type || a.density != b.density || a.E != b.E || a.nu != b.nu || a.yield != b.yield ||
                a.C0 != b.C0 || a.C1 != b.C1)
                return false;
        }
        return true;
    }
    // the same objects in the same order, each at the position this session left it
    bool same_particles(const std::vector<MP*>& mps) const {
        if (mps.size() != mps_.size()) return false;
        for (size_t p = 0; p < mps.size(); ++p) {
            if (mps[p] != mps_[p]) return false;
            for (int k = 0; k < 3; ++k)
                if (mps[p]->d3_Position[k] != pos_[3 * p + k]) return false;
        }
        return true;
    }
    void remember(const std::vector<MP*>& mps) {
        mps_.assign(mps.begin(), mps.end());
        pos_.resize(3 * mps.size());
        for (size_t p = 0; p < mps.size(); ++p)
            for (int k = 0; k < 3; ++k) pos_[3 * p + k] = mps[p]->d3_Position[k];
    }

    int form_;
    mpm_ctx* ctx_ = nullptr;
    mpm_grid_desc grid_ = {};
    bool stale_ = true;
    long long uploads_ = 0;
    const char* err_ = "";
    std::vector<mpm_material> mats_;
    std::vector<const MP*> mps_;
    std::vector<double> pos_;
    std::vector<double> tl_t_, tl_v_;
    ParticleArrays P_;
    NodeArrays G_;
};

}  // namespace mpm_dropin
