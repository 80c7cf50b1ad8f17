// cuda_solver.hpp -- C++ host side above the C ABI (include/fea_gpu.h).
//
// Mirrors the reference's solver layer so that application code written
// against it ports unchanged:
//   Solver        include/FEM/Solver.hpp:8-14  (advance_time, clear_values,
//                 has_numerical_instability over a shared FEMContext)
//   FEMContext    include/FEM/FEMContext.hpp:26-56 (surface, parameters,
//                 equation, boundary_condition, idx_map)
//   Surface       include/Utils/Surface.hpp:36-40,47 (vertices, triangles,
//                 on_boundary, values, num_boundary_points)
// CUDASolver follows CPUSolver's per-step contract (CPUSolver.cpp:64-146):
// it reads surface->values, advances one step on the GPU and writes the
// field back (Dirichlet points read 0).  Errors surface as
// std::runtime_error, as the reference's mesh loading does
// (Surface.cpp:40-41, 59-74).
#pragma once

#include <array>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "fea_gpu.h"

namespace fea {

enum class Equation { Heat = FEA_HEAT, Wave = FEA_WAVE, Advection_Diffusion = FEA_ADVECTION_DIFFUSION,
                      Reaction_Diffusion = FEA_REACTION_DIFFUSION };
enum class BoundaryCondition { Dirichlet = FEA_DIRICHLET, Neumann = FEA_NEUMANN };

enum class MeshType { Open = FEA_MESH_OPEN, Closed = FEA_MESH_CLOSED, Mirrored = FEA_MESH_MIRRORED };

struct Surface {
    std::vector<std::array<float, 3>> vertices;
    std::vector<std::array<float, 3>> normals;  // Surface::normals (Surface.cpp:91-102)
    std::vector<std::array<uint32_t, 3>> triangles;
    std::vector<bool> on_boundary;  // empty: detected on the device
    std::vector<float> values;
    std::vector<std::array<float, 3>> calculated_normals;  // the smooth-normals output
    int num_boundary_points = 0;
};

struct FEMContext {
    std::shared_ptr<Surface> surface;
    fea_params parameters{};  // the four EquationParameters structs + extensions
    Equation equation = Equation::Wave;                            // FEMContext.hpp:31
    BoundaryCondition boundary_condition = BoundaryCondition::Dirichlet;  // FEMContext.hpp:32
    std::vector<int> idx_map;

    FEMContext() { fea_params_default(&parameters); }
};

class Solver {
public:
    std::shared_ptr<FEMContext> fem_ctx;

    virtual void advance_time() = 0;
    virtual void clear_values() = 0;
    virtual bool has_numerical_instability() = 0;
    virtual ~Solver() = default;
};

inline void check(int rc, const char* what) {
    if (rc != FEA_OK) throw std::runtime_error(std::string(what) + ": " + fea_last_error());
}

class CUDASolver : public Solver {
public:
    int precision;

    explicit CUDASolver(std::shared_ptr<FEMContext> ctx, int precision_ = FEA_FP32) : precision(precision_) {
        fem_ctx = std::move(ctx);
        init();
    }
    ~CUDASolver() override { fea_destroy(handle_); }
    CUDASolver(const CUDASolver&) = delete;
    CUDASolver& operator=(const CUDASolver&) = delete;

    // FEMContext::init_from_surface / update_boundary_conditions: assemble on the device.
    void init() {
        fea_destroy(handle_);
        handle_ = nullptr;
        const Surface& s = *fem_ctx->surface;
        std::vector<uint8_t> ob;
        if (!s.on_boundary.empty()) {
            ob.resize(s.on_boundary.size());
            for (size_t i = 0; i < ob.size(); i++) ob[i] = s.on_boundary[i] ? 1 : 0;
        }
        fea_params p = fem_ctx->parameters;
        p.equation = static_cast<int>(fem_ctx->equation);
        check(fea_create(reinterpret_cast<const float*>(s.vertices.data()), (int64_t)s.vertices.size(),
                         reinterpret_cast<const uint32_t*>(s.triangles.data()), (int64_t)s.triangles.size(),
                         ob.empty() ? nullptr : ob.data(), static_cast<int>(fem_ctx->boundary_condition),
                         precision, &p, &handle_),
              "fea_create");
        bc_ = fem_ctx->boundary_condition;
        fea_info info{};
        check(fea_get_info(handle_, &info), "fea_get_info");
        fem_ctx->surface->num_boundary_points = (int)info.num_boundary_points;
        fem_ctx->idx_map.assign(s.vertices.size(), -1);
        check(fea_get_idx_map(handle_, fem_ctx->idx_map.data(), nullptr), "fea_get_idx_map");
        applied_ = p;
    }

    void advance_time() override {
        sync_context();
        Surface& s = *fem_ctx->surface;
        check(fea_set_values(handle_, s.values.data()), "fea_set_values");
        check(fea_advance_time(handle_, 1), "fea_advance_time");
        check(fea_get_values(handle_, s.values.data()), "fea_get_values");
    }

    void clear_values() override { check(fea_clear_values(handle_), "fea_clear_values"); }

    bool has_numerical_instability() override {
        int out = 0;
        check(fea_has_numerical_instability(handle_, &out), "fea_has_numerical_instability");
        return out != 0;
    }

    // Surface::calculate_normals (Surface.cpp:287-306) on the solver's field.
    void calculate_normals(float vertex_extrusion) {
        Surface& s = *fem_ctx->surface;
        s.calculated_normals.resize(s.vertices.size());
        check(fea_smooth_normals(handle_, reinterpret_cast<const float*>(s.normals.data()), vertex_extrusion,
                                 reinterpret_cast<float*>(s.calculated_normals.data())),
              "fea_smooth_normals");
    }

    // Surface::export_to_ply (Surface.cpp:138-285); coeffs: the color map's
    // 7 RGB coefficients (nullptr: gray).
    void export_to_ply(const char* path, float vertex_extrusion = 0.25f, float threshold = 0.0f,
                       MeshType mesh_type = MeshType::Open, const float* coeffs = nullptr) {
        const Surface& s = *fem_ctx->surface;
        check(fea_export_ply(handle_, path, reinterpret_cast<const float*>(s.normals.data()), vertex_extrusion,
                             threshold, static_cast<int>(mesh_type), coeffs),
              "fea_export_ply");
    }

    fea_solver* handle() { return handle_; }

private:
    fea_solver* handle_ = nullptr;
    fea_params applied_{};
    BoundaryCondition bc_ = BoundaryCondition::Dirichlet;

    // Parameters and BC are read from the context every step, as CPUSolver
    // reads fem_ctx->parameters each advance_time.
    void sync_context() {
        if (fem_ctx->boundary_condition != bc_) {
            check(fea_set_boundary_condition(handle_, static_cast<int>(fem_ctx->boundary_condition)),
                  "fea_set_boundary_condition");
            bc_ = fem_ctx->boundary_condition;
            fem_ctx->idx_map.assign(fem_ctx->surface->vertices.size(), -1);
            check(fea_get_idx_map(handle_, fem_ctx->idx_map.data(), nullptr), "fea_get_idx_map");
        }
        fea_params p = fem_ctx->parameters;
        p.equation = static_cast<int>(fem_ctx->equation);
        if (std::memcmp(&p, &applied_, sizeof(p)) != 0) {
            check(fea_set_params(handle_, &p), "fea_set_params");
            applied_ = p;
        }
    }
};

}  // namespace fea
