// sim_cloth: command-line cloth simulation on the GB300 PD solver.
//
// Same command line as the reference driver (src/tools/sim_cloth.cpp:107-161):
//   sim_cloth <nrows> <ncols> <size> [--steps n] [--dt t] [--pin top|corners]
//             [--stiffness k] [--bend k] [--iter n] [--type 0-3] [--gravity g]
//             [--damping d] [--stretch-backend gpu-current] [--export dir] [--verbose]
// plus [--mode consistent|literal] [--rho r] [--tol t].  Energy printout
// (src/tools/sim_cloth.cpp:64-105) and ASCII PLY export (:20-61) as the
// reference; the solve runs through the cloth_pdg shim over the C ABI.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "pd_solver.hpp"

using namespace cloth_pdg;

static void export_ply(const ClothMesh& mesh, const char* path)
{
    FILE* fp = std::fopen(path, "w");
    if (!fp) { std::fprintf(stderr, "Failed to open %s for writing\n", path); return; }
    std::fprintf(fp, "ply\nformat ascii 1.0\nelement vertex %d\n", mesh.num_verts);
    std::fprintf(fp, "property float x\nproperty float y\nproperty float z\n");
    std::fprintf(fp, "element face %d\nproperty list uchar int vertex_indices\nend_header\n", mesh.num_tris);
    for (int i = 0; i < mesh.num_verts; ++i)
        std::fprintf(fp, "%f %f %f\n", mesh.pos_cpu[3 * i], mesh.pos_cpu[3 * i + 1], mesh.pos_cpu[3 * i + 2]);
    for (int t = 0; t < mesh.num_tris; ++t)
        std::fprintf(fp, "3 %d %d %d\n", mesh.triangles[3 * t], mesh.triangles[3 * t + 1], mesh.triangles[3 * t + 2]);
    std::fclose(fp);
}

// kinetic + gravitational potential energy of the downloaded state
static double energy(const ClothMesh& mesh, const std::vector<float>& m, float gravity)
{
    double ke = 0.0, pe = 0.0;
    for (int i = 0; i < mesh.num_verts; ++i) {
        const double vx = mesh.vel_cpu[3 * i], vy = mesh.vel_cpu[3 * i + 1], vz = mesh.vel_cpu[3 * i + 2];
        ke += 0.5 * m[i] * (vx * vx + vy * vy + vz * vz);
        pe += m[i] * (-gravity) * mesh.pos_cpu[3 * i + 1];
    }
    return ke + pe;
}

static void usage(const char* prog)
{
    std::fprintf(stderr, "Usage: %s <nrows> <ncols> <size> [options]\n\n", prog);
    std::fprintf(stderr,
                 "Options:\n"
                 "  --steps <n>      Simulation steps        (default: 100)\n"
                 "  --dt <t>         Time step               (default: 0.01)\n"
                 "  --pin <mode>     top | corners           (default: top)\n"
                 "  --stiffness <k>  Stretch stiffness       (default: 1.0)\n"
                 "  --bend <k>       Bend stiffness          (default: 0 = off)\n"
                 "  --iter <n>       PD iterations/frame     (default: 50)\n"
                 "  --type <n>       Mesh type 0-3           (default: 3)\n"
                 "  --gravity <g>    Gravitational accel     (default: -9.8)\n"
                 "  --damping <d>    Velocity damping 0-1    (default: 0)\n"
                 "  --stretch-backend <b>  gpu-current       (default: gpu-current)\n"
                 "  --export <dir>   Export PLY frames\n"
                 "  --verbose        Per-frame energy output\n"
                 "  --mode <m>       consistent | literal    (default: consistent)\n"
                 "  --rho <r>        Chebyshev rho           (default: 0.9)\n"
                 "  --tol <t>        Stop at this relative residual (default: off)\n");
}

int main(int argc, char** argv)
{
    if (argc < 4) { usage(argv[0]); return 1; }
    const int nrows = std::atoi(argv[1]), ncols = std::atoi(argv[2]);
    const float size = (float)std::atof(argv[3]);
    int steps = 100, iterations = 50, mesh_type = 3;
    float dt = 0.01f, stiffness = 1.0f, bend = 0.0f, gravity = -9.8f, damping = 0.0f, rho = 0.9f, tol = 0.f;
    std::string pin_mode = "top", backend = "gpu-current", export_dir, mode = "consistent";
    bool verbose = false;
    for (int i = 4; i < argc; ++i) {
        const std::string a = argv[i];
        const bool has = i + 1 < argc;
        if (a == "--steps" && has) steps = std::atoi(argv[++i]);
        else if (a == "--dt" && has) dt = (float)std::atof(argv[++i]);
        else if (a == "--pin" && has) pin_mode = argv[++i];
        else if (a == "--stiffness" && has) stiffness = (float)std::atof(argv[++i]);
        else if (a == "--bend" && has) bend = (float)std::atof(argv[++i]);
        else if (a == "--iter" && has) iterations = std::atoi(argv[++i]);
        else if (a == "--type" && has) mesh_type = std::atoi(argv[++i]);
        else if (a == "--gravity" && has) gravity = (float)std::atof(argv[++i]);
        else if (a == "--damping" && has) damping = (float)std::atof(argv[++i]);
        else if (a == "--stretch-backend" && has) backend = argv[++i];
        else if (a == "--export" && has) export_dir = argv[++i];
        else if (a == "--verbose") verbose = true;
        else if (a == "--mode" && has) mode = argv[++i];
        else if (a == "--rho" && has) rho = (float)std::atof(argv[++i]);
        else if (a == "--tol" && has) tol = (float)std::atof(argv[++i]);
    }
    if (backend != "gpu-current") {
        std::fprintf(stderr, "stretch backend '%s' is not available: this solver runs on the GPU only\n", backend.c_str());
        return 2;
    }
    std::printf("=== PD Cloth Simulation ===\n");
    std::printf("Grid: %d x %d, size: %.4f, type: %d\n", nrows, ncols, size, mesh_type);
    std::printf("Steps: %d, dt: %.4f, iter: %d\n", steps, dt, iterations);
    std::printf("stiffness: %.3f, bend: %.4f, damping: %.3f, pin: %s, backend: %s, mode: %s\n", stiffness, bend,
                damping, pin_mode.c_str(), backend.c_str(), mode.c_str());
    try {
        ClothMesh mesh;
        generate_square_cloth(nrows, ncols, size, mesh_type, mesh);
        MeshTopology topo = MeshTopology::build(mesh);
        std::printf("Mesh: %d vertices, %d triangles, %zu edges (%d inner)\n", mesh.num_verts, mesh.num_tris,
                    topo.edges.size(), topo.num_inner_edges());
        SimConstraints sim;
        sim.build_stretch(mesh, stiffness);
        if (bend > 0.f) sim.build_bend(mesh, topo, bend);
        Constraints pins;
        if (pin_mode == "top") pins.pin_top_row(mesh, ncols);
        else if (pin_mode == "corners") pins.pin_corners(mesh, ncols);
        std::printf("Pinned vertices: %zu, bend constraints: %d\n", pins.pinned_indices.size(), sim.num_bend_cons);

        PDSolverConfig cfg;
        cfg.dt = dt; cfg.max_iterations = iterations; cfg.gravity = gravity; cfg.damping = damping;
        cfg.stretch_stiffness = stiffness; cfg.bend_stiffness = bend; cfg.rho = rho;
        cfg.use_tolerance = tol > 0.f; cfg.tolerance = tol;
        cfg.reference_literal = mode == "literal";
        PDSolver solver(cfg, mesh, sim);
        const std::vector<float> m = mesh.mass();
        if (!export_dir.empty()) {
            const std::string fn = export_dir + "/frame_0000.ply";
            export_ply(mesh, fn.c_str());
        }
        std::printf("\nSimulating...\nInitial energy: %.6f\n", energy(mesh, m, gravity));
        const int every = std::max(1, steps / 10);
        for (int s = 1; s <= steps; ++s) {
            solver.step(mesh, sim, pins);
            if ((verbose && s % 10 == 0) || (!export_dir.empty() && s % every == 0)) solver.download(mesh);
            if (verbose && s % 10 == 0) {
                const pdg_frame_stats& st = solver.last_stats();
                std::printf("Step %d: Energy = %.6f  (sweeps %d, rel. residual %.3e)\n", s, energy(mesh, m, gravity),
                            st.iterations, st.rel_residual);
            }
            if (!export_dir.empty() && s % every == 0) {
                char fn[512];
                std::snprintf(fn, sizeof(fn), "%s/frame_%04d.ply", export_dir.c_str(), s / every);
                export_ply(mesh, fn);
            }
        }
        solver.download(mesh);
        std::printf("Final energy: %.6f\n", energy(mesh, m, gravity));
        if (!export_dir.empty()) {
            const std::string fn = export_dir + "/frame_final.ply";
            export_ply(mesh, fn.c_str());
            std::printf("\nExported frames to %s/\n", export_dir.c_str());
        }
    } catch (const Error& e) {
        std::fprintf(stderr, "error %d: %s\n", e.code, e.what());
        return 3;
    }
    std::printf("\nSimulation complete.\n");
    return 0;
}
