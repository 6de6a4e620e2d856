// Shim for the reference build only (oracle/_ref): declaration-compatible OpenGLGrid2D
// (include/simulation/data/OpenGLGrid2D.h) whose bodies abort; the reference's CPU solver files name it
// only inside their OpenGL solver classes, which the oracle never constructs.
#pragma once
#include <cstdlib>
#include "simulation/data/IGrid.h"
#include "simulation/data/StorageBuffer.h"  // the reference's own header; no-op bodies in ref_driver.cpp
class ScalField2D; class VecField2D;
class OpenGLGrid2D final : public IGrid2D {
public:
    OpenGLGrid2D() : IGrid2D(0, 0) {}
    ~OpenGLGrid2D() override {}
    VecField2D& vel() override { std::abort(); }
    ScalField2D& rho() override { std::abort(); }
    ScalField2D& gamma() override { std::abort(); }
    ScalField2D& beta() override { std::abort(); }
    ScalField2D& divergence() override { std::abort(); }
    ScalField2D& pressure() override { std::abort(); }
    VecField2D& forces() override { std::abort(); }
    ScalField2D& boundary() override { std::abort(); }
    StorageBuffer& gpuRho() const { std::abort(); }
    StorageBuffer& gpuBoundary() const { std::abort(); }
    StorageBuffer& gpuPressure() const { std::abort(); }
    StorageBuffer& gpuDivergence() const { std::abort(); }
};
