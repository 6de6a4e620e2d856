// Shim for the reference build only (oracle/_ref): only the RenderData3D struct of the reference's
// SimulationDisplay3D (include/simulation/display/SimulationDisplay3D.h), which CPUSimulator3D returns.
#pragma once
class IGrid3D; class Renderer3D;
class SimulationDisplay3D {
public:
    struct RenderData3D { const int dim = 3; IGrid3D* grid; Renderer3D* renderer; };
};
