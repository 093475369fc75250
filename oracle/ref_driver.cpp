// Headless driver for the reference solver, compiled against the reference's
// own sources (see oracle/build_ref.sh).  Test infrastructure only.
//
// It loads an MPMSNAP1 state into a PhysicsEngine (through a subclass, which
// can reach the protected state in PhysicsEngine.h:81-120), advances it with
// the reference's own runSimulation_Classic_DoublePass_MPLocks or
// runSimulation_Classic_DoublePass_MPLocks_Contact
// (PhysicsEngine_runSimulation_Classic_DoublePass_MPLocks.cpp:439-815,
//  PhysicsEngine_runSimulation_Classic_DoublePass_MPLocks_Contact.cpp:4-566),
// one call per step, and writes the resulting state back out.
//
// Built with -DMPM_REF_LARGE_STRAIN (ref_seq_ls), the non-contact loop runs
// the reference's large-strain pass 2; the output state records contact = 2.
// The elastic deformation gradient is always written out.
//
// usage: ref_driver <in.snap> <out.snap> <steps> <contact 0|1> [timing 0|1]
#include "PhysicsEngine.h"

#include <chrono>
#include <cstdio>
#include <cstdlib>

extern "C" {
#include "mpm_snapshot.h"
}

class HeadlessEngine : public PhysicsEngine {
   public:
    std::vector<Material_BC*> mats;

    void load(const mpmsnap& s) {
        glm::dvec3 length(s.h.length[0], s.h.length[1], s.h.length[2]);
        glm::ivec3 cells(s.h.cells[0], s.h.cells[1], s.h.cells[2]);
        glm::dvec3 cell = length / glm::dvec3(cells);
        for (int t = 0; t < _MAX_N_THREADS; ++t) {
            mpm_GP_Mediator_Thread[t].d3_Length_Grid = length;
            mpm_GP_Mediator_Thread[t].d3_Length_Cell = cell;
            mpm_GP_Mediator_Thread[t].i3_Cells = cells;
            mpm_GP_Mediator_Thread[t].i3_Node_Count = cells + glm::ivec3(1, 1, 1);
        }
        d3_Length_World = length;
        GridPoint_Factory gpf;
        allGridPoint = gpf.createGrid(length, cells);
        if (allGridPoint.size() != s.h.n_nodes) {
            fprintf(stderr, "node count mismatch %zu vs %llu\n", allGridPoint.size(), (unsigned long long)s.h.n_nodes);
            exit(3);
        }
        for (size_t i = 0; i < allGridPoint.size(); ++i) {
            GridPoint* g = allGridPoint[i];
            g->b3_Fixed = glm::bvec3((s.fixed[i] & MPM_NF_FIX_X) != 0, (s.fixed[i] & MPM_NF_FIX_Y) != 0,
                                     (s.fixed[i] & MPM_NF_FIX_Z) != 0);
            g->d_FrictionCoefficient = s.friction[i];
            g->d_Mass = s.g_mass[i];
            for (int k = 0; k < 3; ++k) {
                g->d3_Momentum[k] = s.g_mom[3 * i + k];
                g->d3_Velocity[k] = s.g_vel[3 * i + k];
                g->d3_Force[k] = s.g_force[3 * i + k];
                g->d3_Force_Temp[k] = s.g_force_temp[3 * i + k];
                g->d3_MassGradient[k] = s.g_mass_gradient[3 * i + k];
            }
            g->b_Active = (s.g_state[i] & MPM_NS_ACTIVE) != 0;
            g->b_Contact = (s.g_state[i] & MPM_NS_CONTACT) != 0;
            g->b_Contact_Positive = (s.g_state[i] & MPM_NS_POSITIVE) != 0;
            g->b_Contact_Negative = (s.g_state[i] & MPM_NS_NEGATIVE) != 0;
        }
        v_GridPoint_Lock.resize(allGridPoint.size());
        for (size_t i = 0; i < v_GridPoint_Lock.size(); ++i) {
            v_GridPoint_Lock[i] = new omp_lock_t;
            omp_init_lock(v_GridPoint_Lock[i]);
        }
        for (uint32_t m = 0; m < s.h.n_materials; ++m) {
            Material_BC* mat = new Material_BC;
            mat->i_ID = m;
            mat->i_MaterialType = (unsigned)s.materials[m].type;
            mat->d_Density = s.materials[m].density;
            mat->d_ElasticModulus = s.materials[m].E;
            mat->d_PoissonRatio = s.materials[m].nu;
            mat->d_YieldStress = s.materials[m].yield;
            mat->d_Hardening_Isotropic_C0 = s.materials[m].C0;
            mat->d_Hardening_Isotropic_C1 = s.materials[m].C1;
            v_allMaterial.push_back(mat);
        }
        allMaterialPoint.reserve(s.h.n_particles);
        for (uint64_t p = 0; p < s.h.n_particles; ++p) {
            MaterialPoint_BC* mp = new MaterialPoint_Classic_CC();
            mp->i_ID = (unsigned)p;
            mp->p_Material = (s.material[p] >= 0 && (uint32_t)s.material[p] < s.h.n_materials) ? v_allMaterial[s.material[p]] : NULL;
            for (int k = 0; k < 3; ++k) {
                mp->d3_Position[k] = s.pos[3 * p + k];
                mp->d3_Velocity[k] = s.vel[3 * p + k];
                mp->d3_Force_External[k] = s.fext[3 * p + k];
                mp->d3_MassGradient[k] = s.mp_mass_gradient[3 * p + k];
            }
            mp->d_Mass = s.mass[p];
            mp->d_Volume = s.vol[p];
            mp->d_Volume_Initial = s.vol0[p];
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) {
                    mp->d33_DeformationGradient[c][r] = s.F[9 * p + 3 * c + r];
                    mp->d33_DeformationGradient_Elastic[c][r] = s.F_elastic[9 * p + 3 * c + r];
                }
            for (int k = 0; k < 6; ++k) {
                mp->d6_Stress[k] = s.stress[6 * p + k];
                mp->d6_Strain[k] = s.strain[6 * p + k];
                mp->d6_Strain_Plastic[k] = s.eps_p[6 * p + k];
                mp->d6_Strain_Rate[k] = s.strain_rate[6 * p + k];
            }
            mp->d_Energy_Strain = s.e_strain[p];
            mp->d_Energy_Strain_MaxHistory = s.e_strain_max[p];
            mp->d_Energy_Strain_TimeIntegral = s.e_strain_ti[p];
            mp->d_Energy_Plastic = s.e_plastic[p];
            mp->d_BackStress_Isotropic = s.backstress[p];
            uint8_t fl = s.pflags[p];
            mp->b3_DisplacementControl = glm::bvec3((fl & MPM_PF_DC_X) != 0, (fl & MPM_PF_DC_Y) != 0, (fl & MPM_PF_DC_Z) != 0);
            mp->b_DisplacementControl = (fl & MPM_PF_DC_SKIP) != 0;
            mp->b_Surface = (fl & MPM_PF_SURFACE) != 0;
            mp->f_DisplacementControl_Multiplier = s.dc_mult[p];
            allMaterialPoint.push_back(mp);
        }
        for (uint32_t i = 0; i < s.h.n_dc; ++i) v_MarkedMaterialPoints_Displacement_Control.push_back(allMaterialPoint[s.dc_list[i]]);
        for (uint32_t i = 0; i < s.h.n_timeline; ++i)
            m_TimeLine.addTimePoint(s.tl_time[i], glm::dvec3(s.tl_vel[3 * i], s.tl_vel[3 * i + 1], s.tl_vel[3 * i + 2]));
        d_Time = s.h.time;
        i_TimeCycle = (int)s.h.step;
        d_TimeIncrement_Maximum = s.h.dt_max;
        d_Mass_Minimum = s.h.mass_min;
        d_DampingCoefficient = s.h.damping;
        d_TimeEnd = 1.0e300;
        d_TimeConsole_Interval = 1.0e300;
        d_TimeConsole_Last = d_Time;
        str_Log_FileName = "/dev/null";
        a_Runtime.fill(0.0);
    }

    void store(mpmsnap& s) {
        s.h.time = d_Time;
        s.h.step = i_TimeCycle;
        for (size_t i = 0; i < allGridPoint.size(); ++i) {
            GridPoint* g = allGridPoint[i];
            s.g_mass[i] = g->d_Mass;
            for (int k = 0; k < 3; ++k) {
                s.g_mom[3 * i + k] = g->d3_Momentum[k];
                s.g_vel[3 * i + k] = g->d3_Velocity[k];
                s.g_force[3 * i + k] = g->d3_Force[k];
                s.g_force_temp[3 * i + k] = g->d3_Force_Temp[k];
                s.g_mass_gradient[3 * i + k] = g->d3_MassGradient[k];
            }
            s.g_state[i] = (uint8_t)((g->b_Active ? MPM_NS_ACTIVE : 0) | (g->b_Contact ? MPM_NS_CONTACT : 0) |
                                     (g->b_Contact_Positive ? MPM_NS_POSITIVE : 0) |
                                     (g->b_Contact_Negative ? MPM_NS_NEGATIVE : 0));
        }
        for (size_t p = 0; p < allMaterialPoint.size(); ++p) {
            MaterialPoint_BC* mp = allMaterialPoint[p];
            for (int k = 0; k < 3; ++k) {
                s.pos[3 * p + k] = mp->d3_Position[k];
                s.vel[3 * p + k] = mp->d3_Velocity[k];
                s.fext[3 * p + k] = mp->d3_Force_External[k];
                s.mp_mass_gradient[3 * p + k] = mp->d3_MassGradient[k];
            }
            s.mass[p] = mp->d_Mass;
            s.vol[p] = mp->d_Volume;
            s.vol0[p] = mp->d_Volume_Initial;
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) {
                    s.F[9 * p + 3 * c + r] = mp->d33_DeformationGradient[c][r];
                    s.F_elastic[9 * p + 3 * c + r] = mp->d33_DeformationGradient_Elastic[c][r];
                }
            for (int k = 0; k < 6; ++k) {
                s.stress[6 * p + k] = mp->d6_Stress[k];
                s.strain[6 * p + k] = mp->d6_Strain[k];
                s.eps_p[6 * p + k] = mp->d6_Strain_Plastic[k];
                s.strain_rate[6 * p + k] = mp->d6_Strain_Rate[k];
            }
            s.e_strain[p] = mp->d_Energy_Strain;
            s.e_strain_max[p] = mp->d_Energy_Strain_MaxHistory;
            s.e_strain_ti[p] = mp->d_Energy_Strain_TimeIntegral;
            s.e_plastic[p] = mp->d_Energy_Plastic;
            s.backstress[p] = mp->d_BackStress_Isotropic;
        }
    }
};

int main(int argc, char** argv) {
    if (argc < 5) {
        fprintf(stderr, "usage: %s in.snap out.snap steps contact [timing]\n", argv[0]);
        return 2;
    }
    mpmsnap s;
    int rc = mpmsnap_read(argv[1], &s);
    if (rc != 0) {
        fprintf(stderr, "cannot read %s (%d)\n", argv[1], rc);
        return 3;
    }
    int steps = atoi(argv[3]);
    int contact = atoi(argv[4]);
    int timing = argc > 5 ? atoi(argv[5]) : 0;
    HeadlessEngine eng;
    eng.load(s);
    double dt = s.h.dt_max;
    auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < steps; ++i) {
        if (contact)
            eng.runSimulation_Classic_DoublePass_MPLocks_Contact(dt);
        else
            eng.runSimulation_Classic_DoublePass_MPLocks(dt);
    }
    auto t1 = std::chrono::steady_clock::now();
    double sec = std::chrono::duration<double>(t1 - t0).count();
    if (timing)
        fprintf(stderr, "TIMING steps=%d particles=%llu seconds=%.6f updates_per_s=%.6e\n", steps,
                (unsigned long long)s.h.n_particles, sec, (double)steps * (double)s.h.n_particles / sec);
    s.h.contact = (uint32_t)contact;
#ifdef MPM_REF_LARGE_STRAIN
    if (!contact) s.h.contact = 2u;
#endif
    s.h.flags |= MPMSNAP_HAS_FE;
    eng.store(s);
    rc = mpmsnap_write(argv[2], &s);
    mpmsnap_free(&s);
    return rc == 0 ? 0 : 4;
}
