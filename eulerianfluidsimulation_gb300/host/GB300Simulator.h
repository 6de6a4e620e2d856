// GB300Simulator.h — the GB300 backend as a drop-in beside the reference's CPU / OpenGL / CUDA simulators.
//
// Compiled inside the reference tree (include path: the reference's include/ plus this repository's include/),
// these classes implement the reference interfaces
//   ISimulator3D / ISimulator2D  (include/simulation/simulator/ISimulator*.h, ISimulator.h:8-53)
//   IGrid3D / IGrid2D            (include/simulation/data/IGrid.h:10-68)
// over the C ABI of libefs_gb300.so (include/efs_gb300.h).  Like the reference's CudaSimulator3D
// (src/simulation/simulator/CudaSimulator3D.cu:86-98) a step uploads the host fields, runs on the device and
// downloads them, unless DISABLE_UDLOAD is set; the seven stages run as one CUDA graph replay.
#pragma once

#include "simulation/data/IGrid.h"
#include "simulation/data/ScalField2D.h"
#include "simulation/data/ScalField3D.h"
#include "simulation/data/VecField2D.h"
#include "simulation/data/VecField3D.h"
#include "simulation/display/SimulationDisplay2D.h"
#include "simulation/display/SimulationDisplay3D.h"
#include "simulation/simulator/ISimulator2D.h"
#include "simulation/simulator/ISimulator3D.h"

#include "efs_gb300.h"

// The Properties values the step reads (Properties.h:141-162, 186-192) as the C ABI's parameters: what every
// update() and stage call passes to the device backend.
efs_params GB300ParamsFromProperties();

// Host mirrors of the device fields; the accessors hand out the mirrors as the reference's grids do.
class GB300Grid3D final : public IGrid3D {
public:
    GB300Grid3D(unsigned int width, unsigned int height, unsigned int depth);
    ~GB300Grid3D() override;

    VecField3D& vel() override { return _vel; }
    ScalField3D& rho() override { return _rho; }
    ScalField3D& gamma() override { return _gamma; }
    ScalField3D& beta() override { return _beta; }
    ScalField3D& divergence() override { return _divergence; }
    ScalField3D& pressure() override { return _pressure; }
    VecField3D& forces() override { return _forces; }
    ScalField3D& boundary() override { return _boundary; }

private:
    VecField3D _vel, _forces;
    ScalField3D _rho, _gamma, _beta, _divergence, _pressure, _boundary;
};

class GB300Grid2D final : public IGrid2D {
public:
    GB300Grid2D(unsigned int width, unsigned int height);
    ~GB300Grid2D() override;

    VecField2D& vel() override { return _vel; }
    ScalField2D& rho() override { return _rho; }
    ScalField2D& gamma() override { return _gamma; }
    ScalField2D& beta() override { return _beta; }
    ScalField2D& divergence() override { return _divergence; }
    ScalField2D& pressure() override { return _pressure; }
    VecField2D& forces() override { return _forces; }
    ScalField2D& boundary() override { return _boundary; }

private:
    VecField2D _vel, _forces;
    ScalField2D _rho, _gamma, _beta, _divergence, _pressure, _boundary;
};

class GB300Simulator3D final : public ISimulator3D {
public:
    GB300Simulator3D(unsigned int width, unsigned int height, unsigned int depth);
    ~GB300Simulator3D() override;

    void update() override;
    void* getRenderData() override;

    // text of the last failure of the device backend ("" when none)
    const char* lastError() const;

private:
    void vel_decay() override;
    void vel_extrapolate() override;
    void rho_advect() override;
    void rho_sharpen() override;
    void add_force() override;
    void vel_advect() override;
    void project() override;

    void syncParams();
    void upload();
    void download();
    void stage(int s);
    void readStats();

    GB300Grid3D* _grid{};
    efs_ctx* _ctx{};
    SimulationDisplay3D::RenderData3D* _data{};
};

class GB300Simulator2D final : public ISimulator2D {
public:
    GB300Simulator2D(unsigned int width, unsigned int height);
    ~GB300Simulator2D() override;

    void update() override;
    void* getRenderData() override;
    const char* lastError() const;

private:
    void vel_decay() override;
    void vel_extrapolate() override;
    void rho_advect() override;
    void rho_sharpen() override;
    void add_force() override;
    void vel_advect() override;
    void project() override;

    void syncParams();
    void upload();
    void download();
    void stage(int s);
    void readStats();

    GB300Grid2D* _grid{};
    efs_ctx* _ctx{};
    SimulationDisplay2D::RenderData2D* _data{};
};
