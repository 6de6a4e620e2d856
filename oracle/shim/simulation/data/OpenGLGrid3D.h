// Shim for the reference build only (oracle/_ref): declaration-compatible OpenGLGrid3D
// (include/simulation/data/OpenGLGrid3D.h) whose bodies abort; the reference's CPU solver files name it
// only inside their OpenGL solver classes, which the oracle never constructs.
#pragma once
#include <cstdlib>
#include "simulation/data/IGrid.h"
#include "simulation/data/StorageBuffer.h"  // the reference's own header; no-op bodies in ref_driver.cpp
class ScalField3D; class VecField3D;
class OpenGLGrid3D final : public IGrid3D {
public:
    OpenGLGrid3D() : IGrid3D(0, 0, 0) {}
    ~OpenGLGrid3D() override {}
    VecField3D& vel() override { std::abort(); }
    ScalField3D& rho() override { std::abort(); }
    ScalField3D& gamma() override { std::abort(); }
    ScalField3D& beta() override { std::abort(); }
    ScalField3D& divergence() override { std::abort(); }
    ScalField3D& pressure() override { std::abort(); }
    VecField3D& forces() override { std::abort(); }
    ScalField3D& boundary() override { std::abort(); }
    StorageBuffer& gpuRho() const { std::abort(); }
    StorageBuffer& gpuBoundary() const { std::abort(); }
    StorageBuffer& gpuPressure() const { std::abort(); }
    StorageBuffer& gpuDivergence() const { std::abort(); }
};
