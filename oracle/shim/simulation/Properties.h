// Shim for the reference build only (oracle/_ref).  The reference's Properties singleton
// (include/simulation/Properties.h) needs nlohmann/json and ImGui, both absent.  This header keeps the same
// macro names, token names, enums and typed get/set/add calls, stores the values in two plain arrays, and
// lets the harness install a hook that supplies SOLVER_THRESHOLD (used to turn the reference's absolute
// r.r threshold into a relative-residual one).
#pragma once
#include <type_traits>
#include <vector>
#include "util/Logger.h"

#define PROPERTY(name, type) Properties::Get()->getPropertyValue<type>(Properties::name)
#define PROPERTY_I(name) PROPERTY(name, int)
#define PROPERTY_UI(name) PROPERTY(name, unsigned int)
#define PROPERTY_F(name) PROPERTY(name, float)
#define PROPERTY_B(name) PROPERTY(name, bool)
#define SET_PROPERTY(name, value, type) Properties::Get()->setPropertyValue<type>(Properties::name, value)
#define SET_PROPERTY_I(name, value) SET_PROPERTY(name, value, int)
#define SET_PROPERTY_UI(name, value) SET_PROPERTY(name, value, unsigned int)
#define SET_PROPERTY_F(name, value) SET_PROPERTY(name, value, float)
#define SET_PROPERTY_B(name, value) SET_PROPERTY(name, value, bool)
#define ADD_PROPERTY(name, value, type) Properties::Get()->addPropertyValue<type>(Properties::name, value)
#define ADD_PROPERTY_I(name, value) ADD_PROPERTY(name, value, int)
#define ADD_PROPERTY_UI(name, value) ADD_PROPERTY(name, value, unsigned int)
#define ADD_PROPERTY_F(name, value) ADD_PROPERTY(name, value, float)
#define ADD_PROPERTY_B(name, value) ADD_PROPERTY(name, value, bool)

class Properties {
public:
    enum Token : unsigned int {
        SIMULATION_TYPE, SIMULATION_REBUILD, SIMULATION_RESET, SIMULATION_INITIALIZED, SIMULATION_GRID_RESIZED,
        BRUSH_SIZE, LAMBDA_MINUS, LAMBDA_PLUS, ETA, LIQUID_THRESHOLD, RHO_D,
        GRAVITY_FORCE_PHYSICAL, GRAVITY_FORCE, GRAVITY_ENABLED, MAX_FORCEFIELD_CELLS,
        AVLB_SOLVERS, SOLVER_TYPE, SOLVER_CHECK_INTERVAL, MAX_STEPS, SOLVER_THRESHOLD,
        DT, VEL_EXTRAPOLATE_ITER, VEL_DECAY, CELL_SIZE, WIDTH_2D, HEIGHT_2D, WIDTH_3D, HEIGHT_3D, DEPTH_3D,
        INIT_SHAPE, DRAW_MODE, DRAW_VEL_ARROWS, RE_CALC_DIV, COLOR_BG, COLOR_FLUID, COLOR_BOUNDARY, PAUSED,
        SIMULATION_STEPS, MAX_VALUE, TOTAL_RHO, SOLVE_STEPS, SOLVE_ERRORS,
        DISABLE_VEL_DECAY, DISABLE_VEL_EXTRAPOLATE, DISABLE_RHO_SHARPEN, DISABLE_RHO_ADVECT,
        DISABLE_VEL_ADVECT, DISABLE_ADD_FORCE, DISABLE_PROJECT, DISABLE_UDLOAD,
        WARN_N_CELLS, SIMULATION_FRAMES, VP_SCALE, VP_LOCK, VP_WIDTH, VP_HEIGHT, TOKEN_COUNT
    };
    enum SimulatorType { CPU_2D, OPENGL_2D, END_2D_SIMULATIONS = OPENGL_2D, CPU_3D, OPENGL_3D };
    enum InitShape { FULL, HALF, SQUARE, EMPTY };
    enum DrawMode { VELOCITY, DENSITY, DIVERGENCE, PRESSURE, FLUID, GAMMA, BETA, BOUNDARY };
    enum SolverType { EIGEN_CG, EIGEN_BiCGSTAB, SELF_CG, JACOBI, MULTIGRID };

    static Properties* Get() { static Properties p; return &p; }

    template <typename T> T getPropertyValue(unsigned int token) {
        if constexpr (std::is_pointer_v<T>) return static_cast<T>(ptr[token]);
        else if constexpr (std::is_floating_point_v<T>) {
            if (token == SOLVER_THRESHOLD && threshold_hook) return (T)threshold_hook(threshold_ctx);
            return (T)num[token];
        }
        else if constexpr (std::is_enum_v<T>) return static_cast<T>((long long)num[token]);
        else return (T)num[token];
    }
    template <typename T> void setPropertyValue(unsigned int token, T value) {
        if constexpr (std::is_pointer_v<T>) ptr[token] = (void*)value;
        else num[token] = (double)value;
    }
    template <typename T> void addPropertyValue(unsigned int token, T value) {
        T cur = getPropertyValue<T>(token);
        cur += value;
        setPropertyValue<T>(token, cur);
    }

    double num[TOKEN_COUNT] = {};
    void* ptr[TOKEN_COUNT] = {};
    float (*threshold_hook)(void*) = nullptr;
    void* threshold_ctx = nullptr;

private:
    Properties() {
        ptr[AVLB_SOLVERS] = new std::vector<SolverType>();
        ptr[SOLVE_ERRORS] = new std::vector<float>();
    }
};
