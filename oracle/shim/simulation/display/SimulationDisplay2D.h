// Shim for the reference build only (oracle/_ref): only the RenderData2D struct of the reference's
// SimulationDisplay2D (include/simulation/display/SimulationDisplay2D.h), which CPUSimulator2D returns.
#pragma once
class IGrid2D;
class SimulationDisplay2D {
public:
    struct RenderData2D { const int dim = 2; IGrid2D* grid; unsigned int textureId; };
};
