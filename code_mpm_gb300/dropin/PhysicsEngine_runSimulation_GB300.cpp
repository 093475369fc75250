// Drop-in replacement for
//   PhysicsEngine_runSimulation_Classic_DoublePass_MPLocks.cpp
//   PhysicsEngine_runSimulation_Classic_DoublePass_MPLocks_Contact.cpp
// of code_MPM: link this file (and libmpm_gb300.so) instead of those two, and
// PhysicsEngine::runSimulation_Classic_DoublePass_MPLocks(double) and
// ::runSimulation_Classic_DoublePass_MPLocks_Contact(double) (PhysicsEngine.h:54-55)
// run on the GPU through the C ABI of include/mpm_gb300.h.
//
// Each PhysicsEngine keeps one engine context resident across its calls
// (mpm_dropin::Session, mpm_dropin.hpp): the first call packs the engine's
// heap objects (allMaterialPoint, allGridPoint, v_allMaterial,
// v_MarkedMaterialPoints_Displacement_Control, m_TimeLine) into the
// structure-of-arrays views and uploads them; later calls upload again only
// when the particle list is not the one the last call left (another count or
// object, or a moved particle), so the viewer's per-frame calls
// (GraphicsEngine_gameLoop.cpp:31,41) go straight to the steps.  The steps
// follow the reference's time chunking (…MPLocks.cpp:449-458) and report to
// the console at its interval (:796-800); at every report and at the end of
// every call every MaterialPoint_BC / GridPoint field is current, so callers
// that read the objects between calls see what the CPU solver would have
// left.  A caller that edits particle fields other than the position, or node
// fields, between calls calls gb300_invalidate(engine) first.
//
// Return value as the reference's (:806-814): 1 once d_Time >= d_TimeEnd,
// else 0.  An engine error prints its message to stderr, drops the engine's
// context (the objects keep the state of the last report or call) and
// returns 1, so the caller's loop stops as at the end of a run.
//
// MPM_DROPIN_FORM=fp32 in the environment selects the chosen form (FP32
// transfers and grid, FP64 positions and energies); the default is the plain
// FP64 form, which matches the reference's results.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <vector>

#include "PhysicsEngine.h"
#include "mpm_dropin.hpp"
#include "mpm_gb300.h"

namespace {

using Session = mpm_dropin::Session<MaterialPoint_BC, GridPoint, Material_BC>;

// one resident session per solver instance, released at exit
std::map<const PhysicsEngine*, std::unique_ptr<Session>>& sessions() {
    static std::map<const PhysicsEngine*, std::unique_ptr<Session>> s;
    return s;
}

int form_from_env() {
    const char* f = std::getenv("MPM_DROPIN_FORM");
    return (f && std::strcmp(f, "fp32") == 0) ? MPM_FORM_FP32 : MPM_FORM_FP64;
}

}  // namespace

// Drop the resident state of `engine`: its next run packs and uploads every object again.
void gb300_invalidate(const PhysicsEngine* engine) {
    auto it = sessions().find(engine);
    if (it != sessions().end()) it->second->invalidate();
}

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
    const double t_start = omp_get_wtime();
    auto& slot = sessions()[self];
    if (!slot) slot.reset(new Session(form_from_env()));
    Session& S = *slot;
    mpm_grid_desc gd = {};
    for (int a = 0; a < 3; ++a) {
        gd.length[a] = geom.d3_Length_Grid[a];
        gd.cells[a] = geom.i3_Cells[a];
    }
    std::vector<double> tv;
    tv.reserve(3 * timeline.v_Velocity.size());
    for (const glm::dvec3& v : timeline.v_Velocity) tv.insert(tv.end(), {v.x, v.y, v.z});
    mpm_dropin::Clock clk{time, cycle, dt_max, mass_min, damping, time_end, console_last, console_interval};
    int rc = S.attach(gd, mps, gps, materials, dc, timeline.v_Time, tv, clk);
    if (rc == MPM_OK) {
        rc = S.run(total, contact, clk, mps, gps, [&]() { (self->*report)(""); });
        runtime += omp_get_wtime() - t_start;
    }
    if (rc < 0) {
        std::fprintf(stderr, "GB300 MPM engine error %d: %s\n", rc, S.error());
        sessions().erase(self);
        return 1;
    }
    if (rc == 1) std::cout << "Analysis complete ..." << std::endl;
    return rc;
}
