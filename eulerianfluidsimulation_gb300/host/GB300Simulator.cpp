// GB300Simulator.cpp — see GB300Simulator.h.
#include "GB300Simulator.h"

#include <cstdio>

#include "simulation/Properties.h"

// The Properties values the step reads (include/simulation/Properties.h:141-162, 186-192), as efs_params.
efs_params GB300ParamsFromProperties() {
    efs_params p;
    efs_params_default(&p);
    p.dt = PROPERTY_F(DT);
    p.gravity_force = PROPERTY_F(GRAVITY_FORCE);
    p.gravity_enabled = PROPERTY_B(GRAVITY_ENABLED) ? 1 : 0;
    p.vel_decay = PROPERTY_F(VEL_DECAY);
    p.lambda_minus = PROPERTY_F(LAMBDA_MINUS);
    p.lambda_plus = PROPERTY_F(LAMBDA_PLUS);
    p.eta = PROPERTY_F(ETA);
    p.liquid_threshold = PROPERTY_F(LIQUID_THRESHOLD);
    p.rho_d = PROPERTY_F(RHO_D);
    p.solver = PROPERTY(SOLVER_TYPE, Properties::SolverType) == Properties::JACOBI ? EFS_SOLVER_JACOBI : EFS_SOLVER_CG;
    p.max_steps = PROPERTY_I(MAX_STEPS);
    p.solver_threshold = PROPERTY_F(SOLVER_THRESHOLD);
    p.tol_rel = 0.f;   // the reference's absolute r.r threshold
    p.cg_variant = EFS_CG_REFERENCE;
    unsigned mask = 0;
    if (PROPERTY_B(DISABLE_VEL_DECAY)) mask |= EFS_STAGE_BIT(EFS_STAGE_VEL_DECAY);
    if (PROPERTY_B(DISABLE_VEL_EXTRAPOLATE)) mask |= EFS_STAGE_BIT(EFS_STAGE_VEL_EXTRAPOLATE);
    if (PROPERTY_B(DISABLE_RHO_SHARPEN)) mask |= EFS_STAGE_BIT(EFS_STAGE_RHO_SHARPEN);
    if (PROPERTY_B(DISABLE_RHO_ADVECT)) mask |= EFS_STAGE_BIT(EFS_STAGE_RHO_ADVECT);
    if (PROPERTY_B(DISABLE_VEL_ADVECT)) mask |= EFS_STAGE_BIT(EFS_STAGE_VEL_ADVECT);
    if (PROPERTY_B(DISABLE_ADD_FORCE)) mask |= EFS_STAGE_BIT(EFS_STAGE_ADD_FORCE);
    if (PROPERTY_B(DISABLE_PROJECT)) mask |= EFS_STAGE_BIT(EFS_STAGE_PROJECT);
    p.disable_mask = mask;
    p.re_calc_div = PROPERTY_B(RE_CALC_DIV) ? 1 : 0;
    return p;
}

namespace {

void report(efs_ctx* ctx, int status, const char* what) {
    if (status != EFS_OK) std::fprintf(stderr, "GB300 backend: %s failed: %s\n", what, efs_last_error(ctx));
}

}  // namespace

// ---------------------------------------------------------------------------------------------------------
// grids: the same construction state as Grid3D / Grid2D (src/simulation/data/Grid3D.cpp:10-48)
// ---------------------------------------------------------------------------------------------------------

GB300Grid3D::GB300Grid3D(unsigned int w, unsigned int h, unsigned int d)
    : IGrid3D(w, h, d), _vel(w, h, d), _forces(w, h, d), _rho(w, h, d), _gamma(w, h, d), _beta(w, h, d),
      _divergence(w, h, d), _pressure(w, h, d), _boundary(w, h, d) {
    _gamma = 1.f;
    for (unsigned z = 0; z < d; z++)
    for (unsigned y = 0; y < h; y++)
    for (unsigned x = 0; x < w; x++)
        if (x == 0 || y == 0 || z == 0 || x == w - 1 || y == h - 1 || z == d - 1) {
            _boundary(x, y, z) = 1.f;
            _rho(x, y, z) = 0.f;
        }
}
GB300Grid3D::~GB300Grid3D() = default;

GB300Grid2D::GB300Grid2D(unsigned int w, unsigned int h)
    : IGrid2D(w, h), _vel(w, h), _forces(w, h), _rho(w, h), _gamma(w, h), _beta(w, h), _divergence(w, h),
      _pressure(w, h), _boundary(w, h) {
    _gamma = 1.f;
    for (unsigned y = 0; y < h; y++)
    for (unsigned x = 0; x < w; x++)
        if (x == 0 || y == 0 || x == w - 1 || y == h - 1) {
            _boundary(x, y) = 1.f;
            _rho(x, y) = 0.f;
        }
}
GB300Grid2D::~GB300Grid2D() = default;

// ---------------------------------------------------------------------------------------------------------
// 3D simulator
// ---------------------------------------------------------------------------------------------------------

GB300Simulator3D::GB300Simulator3D(unsigned int width, unsigned int height, unsigned int depth)
    : ISimulator3D(width, height, depth) {
    availableSolvers(std::vector({Properties::SELF_CG, Properties::JACOBI}));
    _grid = new GB300Grid3D(width, height, depth);
    const efs_params p = GB300ParamsFromProperties();
    report(nullptr, efs_create(3, (int)width, (int)height, (int)depth, &p, &_ctx), "efs_create");
    _data = new SimulationDisplay3D::RenderData3D;
    _data->grid = _grid;
}

GB300Simulator3D::~GB300Simulator3D() {
    efs_destroy(_ctx);
    delete _data;
    delete _grid;
}

void* GB300Simulator3D::getRenderData() { return _data; }
const char* GB300Simulator3D::lastError() const { return _ctx ? efs_last_error(_ctx) : efs_last_error(nullptr); }

void GB300Simulator3D::syncParams() {
    const efs_params p = GB300ParamsFromProperties();
    report(_ctx, efs_set_params(_ctx, &p), "efs_set_params");
}

void GB300Simulator3D::upload() {
    report(_ctx, efs_upload_fields(_ctx, reinterpret_cast<const float*>(_grid->vel().data()), _grid->rho().data(),
                                   _grid->gamma().data(), _grid->boundary().data(),
                                   reinterpret_cast<const float*>(_grid->forces().data())), "upload");
}

void GB300Simulator3D::download() {
    report(_ctx, efs_download_fields(_ctx, reinterpret_cast<float*>(_grid->vel().data()), _grid->rho().data(),
                                     _grid->gamma().data(), _grid->beta().data(), _grid->divergence().data(),
                                     _grid->pressure().data()), "download");
}

void GB300Simulator3D::readStats() {
    efs_stats s;
    if (efs_get_stats(_ctx, &s) != EFS_OK) return;
    SET_PROPERTY_I(SOLVE_STEPS, s.solve_steps);
    if (s.paused) SET_PROPERTY_B(PAUSED, true);
}

// ISimulator::update (ISimulator.h:12-38): all enabled stages as one graph replay between upload and download.
void GB300Simulator3D::update() {
    if (!_ctx) return;
    syncParams();
    if (!PROPERTY_B(DISABLE_UDLOAD)) {
        // upload, one step and download in one call; with page-locked host storage the transfers that no stage
        // waits for overlap the step
        float* vel = reinterpret_cast<float*>(_grid->vel().data());
        report(_ctx, efs_step_host(_ctx, vel, _grid->rho().data(), _grid->gamma().data(), _grid->boundary().data(),
                                   reinterpret_cast<const float*>(_grid->forces().data()), vel, _grid->rho().data(),
                                   _grid->gamma().data(), _grid->beta().data(), _grid->divergence().data(),
                                   _grid->pressure().data()), "efs_step_host");
    } else {
        report(_ctx, efs_step(_ctx, 1), "efs_step");
    }
    readStats();
    ADD_PROPERTY_I(SIMULATION_FRAMES, 1);
}

void GB300Simulator3D::stage(int s) {
    if (!_ctx) return;
    syncParams();
    upload();
    report(_ctx, efs_stage(_ctx, s), "efs_stage");
    download();
    readStats();
}

void GB300Simulator3D::vel_decay() { stage(EFS_STAGE_VEL_DECAY); }
void GB300Simulator3D::vel_extrapolate() { stage(EFS_STAGE_VEL_EXTRAPOLATE); }
void GB300Simulator3D::rho_advect() { stage(EFS_STAGE_RHO_ADVECT); }
void GB300Simulator3D::rho_sharpen() { stage(EFS_STAGE_RHO_SHARPEN); }
void GB300Simulator3D::add_force() { stage(EFS_STAGE_ADD_FORCE); }
void GB300Simulator3D::vel_advect() { stage(EFS_STAGE_VEL_ADVECT); }
void GB300Simulator3D::project() { stage(EFS_STAGE_PROJECT); }

// ---------------------------------------------------------------------------------------------------------
// 2D simulator
// ---------------------------------------------------------------------------------------------------------

GB300Simulator2D::GB300Simulator2D(unsigned int width, unsigned int height) : ISimulator2D(width, height) {
    availableSolvers(std::vector({Properties::SELF_CG, Properties::JACOBI}));
    _grid = new GB300Grid2D(width, height);
    const efs_params p = GB300ParamsFromProperties();
    report(nullptr, efs_create(2, (int)width, (int)height, 1, &p, &_ctx), "efs_create");
    _data = new SimulationDisplay2D::RenderData2D();
    _data->grid = _grid;
}

GB300Simulator2D::~GB300Simulator2D() {
    efs_destroy(_ctx);
    delete _data;
    delete _grid;
}

void* GB300Simulator2D::getRenderData() { return _data; }
const char* GB300Simulator2D::lastError() const { return _ctx ? efs_last_error(_ctx) : efs_last_error(nullptr); }

void GB300Simulator2D::syncParams() {
    const efs_params p = GB300ParamsFromProperties();
    report(_ctx, efs_set_params(_ctx, &p), "efs_set_params");
}

void GB300Simulator2D::upload() {
    report(_ctx, efs_upload_fields(_ctx, reinterpret_cast<const float*>(_grid->vel().data()), _grid->rho().data(),
                                   _grid->gamma().data(), _grid->boundary().data(),
                                   reinterpret_cast<const float*>(_grid->forces().data())), "upload");
}

void GB300Simulator2D::download() {
    report(_ctx, efs_download_fields(_ctx, reinterpret_cast<float*>(_grid->vel().data()), _grid->rho().data(),
                                     _grid->gamma().data(), _grid->beta().data(), _grid->divergence().data(),
                                     _grid->pressure().data()), "download");
}

void GB300Simulator2D::readStats() {
    efs_stats s;
    if (efs_get_stats(_ctx, &s) != EFS_OK) return;
    SET_PROPERTY_I(SOLVE_STEPS, s.solve_steps);
    if (s.paused) SET_PROPERTY_B(PAUSED, true);
}

void GB300Simulator2D::update() {
    if (!_ctx) return;
    syncParams();
    if (!PROPERTY_B(DISABLE_UDLOAD)) {
        // upload, one step and download in one call; with page-locked host storage the transfers that no stage
        // waits for overlap the step
        float* vel = reinterpret_cast<float*>(_grid->vel().data());
        report(_ctx, efs_step_host(_ctx, vel, _grid->rho().data(), _grid->gamma().data(), _grid->boundary().data(),
                                   reinterpret_cast<const float*>(_grid->forces().data()), vel, _grid->rho().data(),
                                   _grid->gamma().data(), _grid->beta().data(), _grid->divergence().data(),
                                   _grid->pressure().data()), "efs_step_host");
    } else {
        report(_ctx, efs_step(_ctx, 1), "efs_step");
    }
    readStats();
    ADD_PROPERTY_I(SIMULATION_FRAMES, 1);
}

void GB300Simulator2D::stage(int s) {
    if (!_ctx) return;
    syncParams();
    upload();
    report(_ctx, efs_stage(_ctx, s), "efs_stage");
    download();
    readStats();
}

void GB300Simulator2D::vel_decay() { stage(EFS_STAGE_VEL_DECAY); }
void GB300Simulator2D::vel_extrapolate() { stage(EFS_STAGE_VEL_EXTRAPOLATE); }
void GB300Simulator2D::rho_advect() { stage(EFS_STAGE_RHO_ADVECT); }
void GB300Simulator2D::rho_sharpen() { stage(EFS_STAGE_RHO_SHARPEN); }
void GB300Simulator2D::add_force() { stage(EFS_STAGE_ADD_FORCE); }
void GB300Simulator2D::vel_advect() { stage(EFS_STAGE_VEL_ADVECT); }
void GB300Simulator2D::project() { stage(EFS_STAGE_PROJECT); }
