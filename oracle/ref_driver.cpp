// ref_driver.cpp — TEST INFRASTRUCTURE ONLY.  Drives the reference's own CPU backend
// (CPUSimulator2D / CPUSimulator3D with CGSolverCPU* / JacobiSolverCPU*, compiled unmodified from the
// reference sources by oracle/Makefile against the shim include directory) through a small C API, so that
// tests can run it on the seeded scenes and compare it with the C restatement in efs_oracle.c.
//
// Scene set-up follows the reference editor: construct the simulator, then write boundary and rho through
// the IGrid accessors (src/core/Editor.cpp:21-38).  One stage is run by disabling the six others and calling
// ISimulator::update() (include/simulation/simulator/ISimulator.h:12-38).
#include <cstring>
#include <cmath>
#include <cfloat>
#include <limits>

#include "simulation/Properties.h"
#include "simulation/data/StorageBuffer.h"
#include "simulation/simulator/CPUSimulator2D.h"
#include "simulation/simulator/CPUSimulator3D.h"
#include "simulation/data/Grid2D.h"
#include "simulation/data/Grid3D.h"
#include "../include/efs_gb300.h"

// No-op bodies for the reference's StorageBuffer declarations (include/simulation/data/StorageBuffer.h);
// only the never-constructed OpenGL solver classes reference them.
StorageBuffer::StorageBuffer(unsigned int) : _id(0), _size(0) {}
StorageBuffer::~StorageBuffer() {}
void StorageBuffer::bind(const int) const {}
void StorageBuffer::clear() const {}
void StorageBuffer::resize(unsigned int) {}
void StorageBuffer::upload(const void*, unsigned int) const {}
void StorageBuffer::download(void*, unsigned int) const {}

namespace {
struct RefSim {
    int dim, w, h, d;
    efs_params prm;
    ISimulator* sim;
    IGrid2D* g2;
    IGrid3D* g3;
};

float* field_ptr(RefSim* r, int f) {
    if (r->dim == 3) {
        IGrid3D* g = r->g3;
        switch (f) {
            case EFS_FIELD_VEL: return reinterpret_cast<float*>(g->vel().data());
            case EFS_FIELD_RHO: return g->rho().data();
            case EFS_FIELD_GAMMA: return g->gamma().data();
            case EFS_FIELD_BETA: return g->beta().data();
            case EFS_FIELD_DIVERGENCE: return g->divergence().data();
            case EFS_FIELD_PRESSURE: return g->pressure().data();
            case EFS_FIELD_FORCES: return reinterpret_cast<float*>(g->forces().data());
            case EFS_FIELD_BOUNDARY: return g->boundary().data();
        }
    } else {
        IGrid2D* g = r->g2;
        switch (f) {
            case EFS_FIELD_VEL: return reinterpret_cast<float*>(g->vel().data());
            case EFS_FIELD_RHO: return g->rho().data();
            case EFS_FIELD_GAMMA: return g->gamma().data();
            case EFS_FIELD_BETA: return g->beta().data();
            case EFS_FIELD_DIVERGENCE: return g->divergence().data();
            case EFS_FIELD_PRESSURE: return g->pressure().data();
            case EFS_FIELD_FORCES: return reinterpret_cast<float*>(g->forces().data());
            case EFS_FIELD_BOUNDARY: return g->boundary().data();
        }
    }
    return nullptr;
}

// SOLVER_THRESHOLD hook: tol_rel^2 * b.b of the current divergence (FP64 sum in cell order), as float.
float threshold_hook(void* ctx) {
    RefSim* r = static_cast<RefSim*>(ctx);
    if (r->prm.tol_rel <= 0) return r->prm.solver_threshold;
    const float* b = field_ptr(r, EFS_FIELD_DIVERGENCE);
    const size_t n = (size_t)r->w * r->h * r->d;
    double bb = 0;
    for (size_t i = 0; i < n; i++) bb += (double)b[i] * (double)b[i];
    float t = (float)((double)r->prm.tol_rel * (double)r->prm.tol_rel * bb);
    return t > 0 ? t : FLT_MIN;
}

void apply_params(RefSim* r, unsigned disable) {
    Properties* P = Properties::Get();
    const efs_params& p = r->prm;
    SET_PROPERTY(SIMULATION_TYPE, r->dim == 3 ? Properties::CPU_3D : Properties::CPU_2D, Properties::SimulatorType);
    SET_PROPERTY(INIT_SHAPE, Properties::EMPTY, Properties::InitShape);
    SET_PROPERTY_F(DT, p.dt);
    SET_PROPERTY_F(GRAVITY_FORCE, p.gravity_force);
    SET_PROPERTY_B(GRAVITY_ENABLED, p.gravity_enabled != 0);
    SET_PROPERTY_F(VEL_DECAY, p.vel_decay);
    SET_PROPERTY_F(LAMBDA_MINUS, p.lambda_minus);
    SET_PROPERTY_F(LAMBDA_PLUS, p.lambda_plus);
    SET_PROPERTY_F(ETA, p.eta);
    SET_PROPERTY_F(LIQUID_THRESHOLD, p.liquid_threshold);
    SET_PROPERTY_F(RHO_D, p.rho_d);
    SET_PROPERTY(SOLVER_TYPE, p.solver == EFS_SOLVER_JACOBI ? Properties::JACOBI : Properties::SELF_CG, Properties::SolverType);
    SET_PROPERTY_I(MAX_STEPS, p.max_steps);
    SET_PROPERTY_F(SOLVER_THRESHOLD, p.solver_threshold);
    SET_PROPERTY_B(RE_CALC_DIV, p.re_calc_div != 0);
    const unsigned toks[7] = {Properties::DISABLE_VEL_DECAY, Properties::DISABLE_VEL_EXTRAPOLATE, Properties::DISABLE_RHO_SHARPEN,
                              Properties::DISABLE_RHO_ADVECT, Properties::DISABLE_VEL_ADVECT, Properties::DISABLE_ADD_FORCE,
                              Properties::DISABLE_PROJECT};
    for (int s = 0; s < 7; s++) P->setPropertyValue<bool>(toks[s], (disable >> s) & 1u);
    P->threshold_hook = threshold_hook;
    P->threshold_ctx = r;
}
}  // namespace

extern "C" {

void* ref_create(int dim, int w, int h, int d, const efs_params* prm) {
    RefSim* r = new RefSim();
    SET_PROPERTY_B(PAUSED, false);
    SET_PROPERTY_I(SOLVE_STEPS, 0);
    SET_PROPERTY_I(SIMULATION_FRAMES, 0);
    r->dim = dim; r->w = w; r->h = h; r->d = (dim == 3) ? d : 1; r->prm = *prm;
    apply_params(r, prm->disable_mask);
    if (dim == 3) {
        auto* s = new CPUSimulator3D(w, h, d);
        r->sim = s;
        r->g3 = static_cast<SimulationDisplay3D::RenderData3D*>(s->getRenderData())->grid;
    } else {
        auto* s = new CPUSimulator2D(w, h);
        r->sim = s;
        r->g2 = static_cast<SimulationDisplay2D::RenderData2D*>(s->getRenderData())->grid;
    }
    return r;
}

void ref_destroy(void* h) { RefSim* r = static_cast<RefSim*>(h); delete r->sim; delete r; }

void ref_set_params(void* h, const efs_params* prm) { RefSim* r = static_cast<RefSim*>(h); r->prm = *prm; apply_params(r, prm->disable_mask); }

float* ref_field(void* h, int f) { return field_ptr(static_cast<RefSim*>(h), f); }

void ref_step(void* h, int n) {
    RefSim* r = static_cast<RefSim*>(h);
    apply_params(r, r->prm.disable_mask);
    for (int i = 0; i < n; i++) r->sim->update();
}

void ref_stage(void* h, int stage) {
    RefSim* r = static_cast<RefSim*>(h);
    apply_params(r, 0x7Fu & ~(1u << stage));
    r->sim->update();
    apply_params(r, r->prm.disable_mask);
}

void ref_stats(void* h, efs_stats* s) {
    (void)h;
    std::memset(s, 0, sizeof(*s));
    s->frames = PROPERTY_I(SIMULATION_FRAMES);
    s->solve_steps = PROPERTY_I(SOLVE_STEPS);
    s->paused = PROPERTY_B(PAUSED) ? 1 : 0;
}

void ref_clear_paused(void) { SET_PROPERTY_B(PAUSED, false); SET_PROPERTY_I(SOLVE_STEPS, 0); }

// QueryNode::update's metric loop (src/simulation/scene/nodes/QueryNode.cpp:52-81) on this simulator's 3D grid:
// the reference's own lines, cut from its source file by oracle/Makefile into _ref/query_loop.inc and compiled
// here with the names they use (position, scale, _only_fluid, grid, w, h, d).  QueryNode.cpp itself cannot be
// compiled: its scene-node headers need GL, JSON and UI types.  out: max, min, avg position, velocity (3 each),
// pressure; returns the count.
long long ref_query_box(void* handle, const float* pos, const float* scl, int only_fluid, float* out) {
    RefSim* r = static_cast<RefSim*>(handle);
    IGrid3D* grid = r->g3;
    const glm::vec3 position(pos[0], pos[1], pos[2]);
    const glm::vec3 scale(scl[0], scl[1], scl[2]);
    const bool _only_fluid = only_fluid != 0;
    const int w = r->w;
    const int h = r->h;
    const int d = r->d;
#include "query_loop.inc"
    const glm::vec3 res[4] = {maxPos, minPos, avgPos, vel};
    for (int k = 0; k < 4; k++)
        for (int c = 0; c < 3; c++) out[3 * k + c] = res[k][c];
    out[12] = pres;
    return count;
}

}  // extern "C"
