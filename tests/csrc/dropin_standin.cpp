// Test driver for the drop-in session (code_mpm_gb300/dropin/mpm_dropin.hpp) on
// stand-in objects: types of this file's own that carry the member names the
// session maps (MaterialPoint_BC.h:25-85, GridPoint.h:6-45, Material_BC.h:13-35,
// with the contact members the reference's headers comment out), so the
// test needs no reference checkout.
//
//   dropin_standin in.snap out.snap steps contact
//
// Builds the objects from the snapshot, then calls the session's run once per
// step (each call one step of dt_max, as a viewer calling every frame would),
// writes the objects back as a snapshot, and prints the session's upload
// count before and after a position nudge between calls.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "mpm_dropin.hpp"
#include "mpm_snapshot.h"

namespace standin {

struct dvec3 {
    double x = 0.0, y = 0.0, z = 0.0;
    double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const double& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
struct bvec3 {
    bool x = false, y = false, z = false;
};
struct dmat3 {  // column-major: m[c][r]
    dvec3 c[3];
    dvec3& operator[](int i) { return c[i]; }
    const dvec3& operator[](int i) const { return c[i]; }
};

struct Material {
    unsigned i_MaterialType = 0;
    double d_Density = 0.0, d_ElasticModulus = 0.0, d_PoissonRatio = 0.0, d_YieldStress = 0.0;
    double d_Hardening_Isotropic_C0 = 0.0, d_Hardening_Isotropic_C1 = 0.0;
};

struct MaterialPoint {
    Material* p_Material = nullptr;
    bool b_DisplacementControl = false;
    bvec3 b3_DisplacementControl;
    float f_DisplacementControl_Multiplier = 1.0f;
    bool b_Surface = false;
    double d_Mass = 0.0, d_Volume = 0.0, d_Volume_Initial = 0.0;
    dvec3 d3_MassGradient, d3_Position, d3_Velocity, d3_Force_External;
    dmat3 d33_DeformationGradient, d33_DeformationGradient_Elastic;
    double d6_Strain[6] = {}, d6_Stress[6] = {}, d6_Strain_Plastic[6] = {}, d6_Strain_Rate[6] = {};
    double d_Energy_Strain = 0.0, d_Energy_Strain_MaxHistory = 0.0, d_Energy_Strain_TimeIntegral = 0.0;
    double d_Energy_Plastic = 0.0, d_BackStress_Isotropic = 0.0;
};

struct GridPoint {
    bool b_Active = false, b_Contact = false, b_Contact_Positive = false, b_Contact_Negative = false;
    bvec3 b3_Fixed;
    double d_FrictionCoefficient = 0.0, d_Mass = 0.0;
    dvec3 d3_MassGradient, d3_Momentum, d3_Velocity, d3_Force, d3_Force_Temp;
};

}  // namespace standin

using namespace standin;
using Session = mpm_dropin::Session<MaterialPoint, GridPoint, Material>;

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s in.snap out.snap steps contact\n", argv[0]);
        return 2;
    }
    mpmsnap s;
    if (mpmsnap_read(argv[1], &s) != 0) return 3;
    const int steps = std::atoi(argv[3]), contact = std::atoi(argv[4]);
    const size_t n = s.h.n_particles, nn = s.h.n_nodes;
    std::vector<Material> mats(s.h.n_materials);
    for (size_t i = 0; i < mats.size(); ++i) {
        const mpmsnap_material& m = s.materials[i];
        mats[i].i_MaterialType = (unsigned)m.type;
        mats[i].d_Density = m.density;
        mats[i].d_ElasticModulus = m.E;
        mats[i].d_PoissonRatio = m.nu;
        mats[i].d_YieldStress = m.yield;
        mats[i].d_Hardening_Isotropic_C0 = m.C0;
        mats[i].d_Hardening_Isotropic_C1 = m.C1;
    }
    std::vector<MaterialPoint> mp(n);
    std::vector<GridPoint> gp(nn);
    for (size_t p = 0; p < n; ++p) {
        MaterialPoint& q = mp[p];
        q.p_Material = s.material[p] >= 0 ? &mats[s.material[p]] : nullptr;
        const uint8_t f = s.pflags[p];
        q.b3_DisplacementControl = {(f & MPM_PF_DC_X) != 0, (f & MPM_PF_DC_Y) != 0, (f & MPM_PF_DC_Z) != 0};
        q.b_DisplacementControl = (f & MPM_PF_DC_SKIP) != 0;
        q.b_Surface = (f & MPM_PF_SURFACE) != 0;
        q.f_DisplacementControl_Multiplier = s.dc_mult[p];
        q.d_Mass = s.mass[p];
        q.d_Volume = s.vol[p];
        q.d_Volume_Initial = s.vol0[p];
        for (int k = 0; k < 3; ++k) {
            q.d3_Position[k] = s.pos[3 * p + k];
            q.d3_Velocity[k] = s.vel[3 * p + k];
            q.d3_Force_External[k] = s.fext[3 * p + k];
            q.d3_MassGradient[k] = s.mp_mass_gradient[3 * p + k];
        }
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) {
                q.d33_DeformationGradient[c][r] = s.F[9 * p + 3 * c + r];
                q.d33_DeformationGradient_Elastic[c][r] = s.F_elastic[9 * p + 3 * c + r];
            }
        for (int k = 0; k < 6; ++k) {
            q.d6_Stress[k] = s.stress[6 * p + k];
            q.d6_Strain[k] = s.strain[6 * p + k];
            q.d6_Strain_Plastic[k] = s.eps_p[6 * p + k];
            q.d6_Strain_Rate[k] = s.strain_rate[6 * p + k];
        }
        q.d_Energy_Strain = s.e_strain[p];
        q.d_Energy_Strain_MaxHistory = s.e_strain_max[p];
        q.d_Energy_Strain_TimeIntegral = s.e_strain_ti[p];
        q.d_Energy_Plastic = s.e_plastic[p];
        q.d_BackStress_Isotropic = s.backstress[p];
    }
    for (size_t i = 0; i < nn; ++i) {
        GridPoint& g = gp[i];
        g.b3_Fixed = {(s.fixed[i] & MPM_NF_FIX_X) != 0, (s.fixed[i] & MPM_NF_FIX_Y) != 0,
                      (s.fixed[i] & MPM_NF_FIX_Z) != 0};
        g.d_FrictionCoefficient = s.friction[i];
        g.d_Mass = s.g_mass[i];
        for (int k = 0; k < 3; ++k) {
            g.d3_Momentum[k] = s.g_mom[3 * i + k];
            g.d3_Velocity[k] = s.g_vel[3 * i + k];
            g.d3_Force[k] = s.g_force[3 * i + k];
            g.d3_Force_Temp[k] = s.g_force_temp[3 * i + k];
            g.d3_MassGradient[k] = s.g_mass_gradient[3 * i + k];
        }
        g.b_Active = (s.g_state[i] & MPM_NS_ACTIVE) != 0;
        g.b_Contact = (s.g_state[i] & MPM_NS_CONTACT) != 0;
        g.b_Contact_Positive = (s.g_state[i] & MPM_NS_POSITIVE) != 0;
        g.b_Contact_Negative = (s.g_state[i] & MPM_NS_NEGATIVE) != 0;
    }
    // the engine's pointer vectors, as PhysicsEngine keeps them
    std::vector<MaterialPoint*> mps(n), dc(s.h.n_dc);
    std::vector<GridPoint*> gps(nn);
    std::vector<Material*> mptr(mats.size());
    for (size_t p = 0; p < n; ++p) mps[p] = &mp[p];
    for (size_t i = 0; i < nn; ++i) gps[i] = &gp[i];
    for (size_t i = 0; i < mats.size(); ++i) mptr[i] = &mats[i];
    for (size_t k = 0; k < dc.size(); ++k) dc[k] = &mp[s.dc_list[k]];
    std::vector<double> tl_t(s.tl_time, s.tl_time + s.h.n_timeline), tl_v(s.tl_vel, s.tl_vel + 3 * s.h.n_timeline);
    mpm_grid_desc gd = {};
    for (int a = 0; a < 3; ++a) {
        gd.length[a] = s.h.length[a];
        gd.cells[a] = s.h.cells[a];
    }
    double time = s.h.time, console_last = -1.0e12;
    int cycle = (int)s.h.step;
    mpm_dropin::Clock clk{time, cycle, s.h.dt_max, s.h.mass_min, s.h.damping, 1.0e300, console_last, 1.0e300};
    Session S(MPM_FORM_FP64);
    int reports = 0;
    auto report = [&]() { ++reports; };
    int rc = S.attach(gd, mps, gps, mptr, dc, tl_t, tl_v, clk);
    if (rc == MPM_OK && steps == 0) rc = S.detach(mps, gps);  // the round trip alone
    for (int k = 0; k < steps && rc >= 0; ++k) {  // one step per call, each call attaching first
        if (k > 0) rc = S.attach(gd, mps, gps, mptr, dc, tl_t, tl_v, clk);
        if (rc == MPM_OK) rc = S.run(s.h.dt_max, contact, clk, mps, gps, report);
    }
    if (rc < 0) {
        std::fprintf(stderr, "engine error %d: %s\n", rc, S.error());
        return 4;
    }
    const long long uploads_run = S.uploads();
    // the objects back into the snapshot
    for (size_t p = 0; p < n; ++p) {
        const MaterialPoint& q = mp[p];
        for (int k = 0; k < 3; ++k) {
            s.pos[3 * p + k] = q.d3_Position[k];
            s.vel[3 * p + k] = q.d3_Velocity[k];
            s.mp_mass_gradient[3 * p + k] = q.d3_MassGradient[k];
        }
        s.vol[p] = q.d_Volume;
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) {
                s.F[9 * p + 3 * c + r] = q.d33_DeformationGradient[c][r];
                s.F_elastic[9 * p + 3 * c + r] = q.d33_DeformationGradient_Elastic[c][r];
            }
        for (int k = 0; k < 6; ++k) {
            s.stress[6 * p + k] = q.d6_Stress[k];
            s.strain[6 * p + k] = q.d6_Strain[k];
            s.eps_p[6 * p + k] = q.d6_Strain_Plastic[k];
            s.strain_rate[6 * p + k] = q.d6_Strain_Rate[k];
        }
        s.e_strain[p] = q.d_Energy_Strain;
        s.e_strain_max[p] = q.d_Energy_Strain_MaxHistory;
        s.e_strain_ti[p] = q.d_Energy_Strain_TimeIntegral;
        s.e_plastic[p] = q.d_Energy_Plastic;
        s.backstress[p] = q.d_BackStress_Isotropic;
    }
    for (size_t i = 0; i < nn; ++i) {
        const GridPoint& g = gp[i];
        s.g_mass[i] = g.d_Mass;
        for (int k = 0; k < 3; ++k) {
            s.g_mom[3 * i + k] = g.d3_Momentum[k];
            s.g_vel[3 * i + k] = g.d3_Velocity[k];
            s.g_force[3 * i + k] = g.d3_Force[k];
            s.g_force_temp[3 * i + k] = g.d3_Force_Temp[k];
            s.g_mass_gradient[3 * i + k] = g.d3_MassGradient[k];
        }
        s.g_state[i] = (uint8_t)((g.b_Active ? MPM_NS_ACTIVE : 0) | (g.b_Contact ? MPM_NS_CONTACT : 0) |
                                 (g.b_Contact_Positive ? MPM_NS_POSITIVE : 0) |
                                 (g.b_Contact_Negative ? MPM_NS_NEGATIVE : 0));
    }
    s.h.time = time;
    s.h.step = cycle;
    s.h.flags |= MPMSNAP_HAS_FE;
    if (mpmsnap_write(argv[2], &s) != 0) return 5;
    // a host edit between calls: the next attach re-packs
    if (n > 0) mp[0].d3_Position[0] += 1.0e-9;
    rc = S.attach(gd, mps, gps, mptr, dc, tl_t, tl_v, clk);
    std::printf("{\"uploads_run\": %lld, \"uploads_after_edit\": %lld, \"reports\": %d, \"rc\": %d}\n", uploads_run,
                S.uploads(), reports, rc);
    mpmsnap_free(&s);
    return rc < 0 ? 6 : 0;
}
