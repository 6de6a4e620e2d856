// dropin_driver.cpp — TEST INFRASTRUCTURE ONLY (tests/test_abi.py builds and runs it where the reference tree is
// present).  Runs the C++ drop-in backend (eulerianfluidsimulation_gb300/host/GB300Simulator.cpp) the way the
// reference application does: the Properties singleton holds the dam-break settings, a simulator is constructed
// through its ISimulator3D interface and update() is called per frame (Application.cpp:76-125).  The
// reference's own CPUSimulator3D runs beside it on the same scene (oracle/_ref/libefs_ref.so holds the
// reference's CPU sources and the field classes).
//
//   dropin_driver params         prints the efs_params the adapter derives from the Properties
//   dropin_driver run N FRAMES   both simulators on an N^3 seeded dam break for FRAMES frames: prints the
//                                relative L2 of rho, vel and pressure between them, SOLVE_STEPS and PAUSED of
//                                each; without a CUDA device it prints the adapter's error text instead
//   dropin_driver reference N FRAMES OUT
//                                the reference's CPUSimulator3D alone, driven the same way: writes to OUT the
//                                int32 values N, FRAMES, SOLVE_STEPS and PAUSED after each frame, the efs_params the
//                                adapter derives from the same Properties (raw bytes), then the float32 fields vel
//                                (x,y,z interleaved), rho, gamma, beta, divergence, pressure after the last frame
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "simulation/Properties.h"
#include "simulation/simulator/CPUSimulator3D.h"
#include "GB300Simulator.h"
#include "efs_scene.h"

namespace {

void dam_properties(int n) {
    Properties* P = Properties::Get();
    SET_PROPERTY(SIMULATION_TYPE, Properties::CPU_3D, Properties::SimulatorType);
    SET_PROPERTY(INIT_SHAPE, Properties::EMPTY, Properties::InitShape);
    SET_PROPERTY_F(DT, 0.004f);
    SET_PROPERTY_F(GRAVITY_FORCE, 9.81f / (1.0f / (float)n));
    SET_PROPERTY_B(GRAVITY_ENABLED, true);
    SET_PROPERTY_F(VEL_DECAY, 0.8f);
    SET_PROPERTY_F(LAMBDA_MINUS, 50.f);
    SET_PROPERTY_F(LAMBDA_PLUS, 10.f);
    SET_PROPERTY_F(ETA, 100.f);
    SET_PROPERTY_F(LIQUID_THRESHOLD, 0.5f);
    SET_PROPERTY_F(RHO_D, 32.f);
    SET_PROPERTY(SOLVER_TYPE, Properties::SELF_CG, Properties::SolverType);
    SET_PROPERTY_I(MAX_STEPS, 2000);
    SET_PROPERTY_F(SOLVER_THRESHOLD, 1e-5f);
    SET_PROPERTY_B(RE_CALC_DIV, false);
    SET_PROPERTY_B(DISABLE_UDLOAD, false);
    const unsigned toks[7] = {Properties::DISABLE_VEL_DECAY, Properties::DISABLE_VEL_EXTRAPOLATE, Properties::DISABLE_RHO_SHARPEN,
                              Properties::DISABLE_RHO_ADVECT, Properties::DISABLE_VEL_ADVECT, Properties::DISABLE_ADD_FORCE,
                              Properties::DISABLE_PROJECT};
    for (int s = 0; s < 7; s++) P->setPropertyValue<bool>(toks[s], s == 0);   // velocity decay off (Dam128.json)
    SET_PROPERTY_B(PAUSED, false);
    SET_PROPERTY_I(SOLVE_STEPS, 0);
    SET_PROPERTY_I(SIMULATION_FRAMES, 0);
}

double rel_l2(const float* a, const float* b, size_t n) {
    double d = 0, r = 0;
    for (size_t i = 0; i < n; i++) { d += ((double)a[i] - b[i]) * ((double)a[i] - b[i]); r += (double)b[i] * b[i]; }
    return r > 0 ? std::sqrt(d / r) : std::sqrt(d);
}

}  // namespace

int main(int argc, char** argv) {
    if (argc >= 2 && std::strcmp(argv[1], "params") == 0) {
        dam_properties(64);
        const efs_params p = GB300ParamsFromProperties();
        std::printf("dt=%.9g gravity_force=%.9g gravity_enabled=%d vel_decay=%.9g lambda_minus=%.9g lambda_plus=%.9g "
                    "eta=%.9g liquid_threshold=%.9g rho_d=%.9g solver=%d max_steps=%d solver_threshold=%.9g tol_rel=%.9g "
                    "disable_mask=%u re_calc_div=%d cg_variant=%d\n",
                    p.dt, p.gravity_force, p.gravity_enabled, p.vel_decay, p.lambda_minus, p.lambda_plus, p.eta,
                    p.liquid_threshold, p.rho_d, p.solver, p.max_steps, p.solver_threshold, p.tol_rel, p.disable_mask,
                    p.re_calc_div, p.cg_variant);
        return 0;
    }
    const bool run = argc == 4 && std::strcmp(argv[1], "run") == 0;
    const bool ref = argc == 5 && std::strcmp(argv[1], "reference") == 0;
    if (!run && !ref) {
        std::fprintf(stderr, "usage: dropin_driver params | run N FRAMES | reference N FRAMES OUT\n");
        return 2;
    }
    const int n = std::atoi(argv[2]), frames = std::atoi(argv[3]);
    if (n < 8 || n > 128 || frames < 1) return 2;
    dam_properties(n);
    const size_t N = (size_t)n * n * n;
    std::vector<float> bnd(N), rho(N);
    efs_scene_dam3d_fill(n, n, n, 4, 4, 3, bnd.data(), rho.data());

    if (ref) {
        CPUSimulator3D cpu(n, n, n);
        IGrid3D* cg = static_cast<SimulationDisplay3D::RenderData3D*>(cpu.getRenderData())->grid;
        std::memcpy(cg->boundary().data(), bnd.data(), N * sizeof(float));
        std::memcpy(cg->rho().data(), rho.data(), N * sizeof(float));
        std::vector<int> steps(frames), paused(frames);
        for (int f = 0; f < frames; f++) {
            SET_PROPERTY_B(PAUSED, false);
            cpu.update();
            steps[f] = PROPERTY_I(SOLVE_STEPS);
            paused[f] = PROPERTY_B(PAUSED) ? 1 : 0;
        }
        const efs_params p = GB300ParamsFromProperties();
        FILE* fo = std::fopen(argv[4], "wb");
        if (!fo) return 1;
        const int head[2] = {n, frames};
        std::fwrite(head, sizeof(int), 2, fo);
        std::fwrite(steps.data(), sizeof(int), frames, fo);
        std::fwrite(paused.data(), sizeof(int), frames, fo);
        std::fwrite(&p, sizeof(p), 1, fo);
        std::fwrite(cg->vel().data(), sizeof(float), 3 * N, fo);
        const float* scal[5] = {cg->rho().data(), cg->gamma().data(), cg->beta().data(), cg->divergence().data(),
                                cg->pressure().data()};
        for (const float* a : scal) std::fwrite(a, sizeof(float), N, fo);
        return std::fclose(fo) == 0 ? 0 : 1;
    }

    GB300Simulator3D gpu(n, n, n);
    CPUSimulator3D cpu(n, n, n);
    IGrid3D* gg = static_cast<SimulationDisplay3D::RenderData3D*>(gpu.getRenderData())->grid;
    IGrid3D* cg = static_cast<SimulationDisplay3D::RenderData3D*>(cpu.getRenderData())->grid;
    if (std::strlen(gpu.lastError()) > 0) {
        std::printf("no-device %s\n", gpu.lastError());
        return 0;
    }
    // the scene written through the IGrid accessors, as the reference editor does (Editor.cpp:21-38)
    std::memcpy(gg->boundary().data(), bnd.data(), N * sizeof(float));
    std::memcpy(gg->rho().data(), rho.data(), N * sizeof(float));
    std::memcpy(cg->boundary().data(), bnd.data(), N * sizeof(float));
    std::memcpy(cg->rho().data(), rho.data(), N * sizeof(float));
    int steps_gpu = 0, steps_cpu = 0;
    bool paused_gpu = false, paused_cpu = false;
    for (int f = 0; f < frames; f++) {
        SET_PROPERTY_B(PAUSED, false);
        gpu.update();
        steps_gpu = PROPERTY_I(SOLVE_STEPS);
        paused_gpu = paused_gpu || PROPERTY_B(PAUSED);
        SET_PROPERTY_B(PAUSED, false);
        cpu.update();
        steps_cpu = PROPERTY_I(SOLVE_STEPS);
        paused_cpu = paused_cpu || PROPERTY_B(PAUSED);
    }
    std::printf("rho=%.3e vel=%.3e pressure=%.3e steps_gpu=%d steps_cpu=%d paused_gpu=%d paused_cpu=%d frames=%d error=%s\n",
                rel_l2(gg->rho().data(), cg->rho().data(), N),
                rel_l2(reinterpret_cast<const float*>(gg->vel().data()), reinterpret_cast<const float*>(cg->vel().data()), 3 * N),
                rel_l2(gg->pressure().data(), cg->pressure().data(), N), steps_gpu, steps_cpu, paused_gpu ? 1 : 0,
                paused_cpu ? 1 : 0, PROPERTY_I(SIMULATION_FRAMES), gpu.lastError());
    return 0;
}
