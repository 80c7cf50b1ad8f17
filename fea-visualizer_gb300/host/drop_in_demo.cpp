// drop_in_demo.cpp -- the reference application's per-frame call sequence
// (Application.cpp:506-565) driven through fea::CUDASolver.
//
//   drop_in_demo <mesh.bin> <out.bin> <equation> <bc> <steps> [out.ply]
//
// mesh.bin: int64 V, int64 T, float xyz[3V], uint32 tri[3T], float values[V].
// out.bin:  float values[V] after `steps` frames, then int32 instability flag.
// Per frame: advance_time(); if has_numerical_instability(): clear_values()
// and stop, as Application::run does (Application.cpp:530-538); then the
// extruded normals (Application.cpp:103).  With out.ply, the surface is
// exported at the end (Surface::export_to_ply, threshold 0, Open).
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>

#include "cuda_solver.hpp"

int main(int argc, char** argv) {
    if (argc < 6) {
        std::cerr << "usage: drop_in_demo mesh.bin out.bin equation bc steps\n";
        return 2;
    }
    std::ifstream in(argv[1], std::ios::binary);
    int64_t V = 0, T = 0;
    in.read(reinterpret_cast<char*>(&V), 8);
    in.read(reinterpret_cast<char*>(&T), 8);
    auto surface = std::make_shared<fea::Surface>();
    surface->vertices.resize(V);
    surface->triangles.resize(T);
    surface->values.resize(V);
    in.read(reinterpret_cast<char*>(surface->vertices.data()), 12 * V);
    in.read(reinterpret_cast<char*>(surface->triangles.data()), 12 * T);
    in.read(reinterpret_cast<char*>(surface->values.data()), 4 * V);
    surface->normals.assign(V, {0.0f, 0.0f, 1.0f});
    if (!in) {
        std::cerr << "short mesh file\n";
        return 2;
    }
    auto ctx = std::make_shared<fea::FEMContext>();
    ctx->surface = surface;
    ctx->equation = static_cast<fea::Equation>(std::atoi(argv[3]));
    ctx->boundary_condition = static_cast<fea::BoundaryCondition>(std::atoi(argv[4]));
    const int steps = std::atoi(argv[5]);
    int unstable = 0;
    try {
        auto cuda = std::make_unique<fea::CUDASolver>(ctx);
        fea::Solver* solver = cuda.get();
        solver->clear_values();
        for (int f = 0; f < steps; f++) {
            solver->advance_time();
            if (solver->has_numerical_instability()) {
                solver->clear_values();
                unstable = 1;
                break;
            }
            cuda->calculate_normals(0.25f);
        }
        if (argc > 6) cuda->export_to_ply(argv[6]);
    } catch (const std::exception& e) {
        std::cerr << "error: " << e.what() << "\n";
        return 1;
    }
    std::ofstream out(argv[2], std::ios::binary);
    out.write(reinterpret_cast<const char*>(surface->values.data()), 4 * V);
    int32_t u = unstable;
    out.write(reinterpret_cast<const char*>(&u), 4);
    std::cout << "frames done, unstable=" << unstable << "\n";
    return 0;
}
