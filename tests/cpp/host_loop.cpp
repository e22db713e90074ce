// host_loop.cpp -- a C++ host that drives the drop-in entry points the way
// the reference's Solver.cpp drives its OpenCL kernels: buffers created once
// from the host vectors (Solver.cpp:232-273), then per RK stage j
// U_Q -> Viscous -> Weno(j) (:377, :440, :521) and the boundary routine
// (:658).  Test program: reads a case (reference layout, raw binary files
// written by the test) from a directory, runs `steps` SSP-RK3 steps, writes
// FLOW back.  No Python in the loop.
//
//   host_loop <dir> <steps> [device|host|rk3]
//     device: device buffers, the three kernels + boundary fill per stage
//     host:   the same calls on the host vectors themselves
//     rk3:    device buffers, one cfd_rk3_step call for all steps
//   dir: meta.txt (n_rows sd_node mach reynolds prandtl t_inf eps viscous les dt
//        n_outlet n_inlet n_boundary n_wall), grid.bin det.bin deter.bin
//        metric.bin flow.bin, outlet.bin inlet.bin boundary.bin wall.bin
//   writes dir/flow_out.bin
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "cfd_rhs.h"

namespace {

template <class T>
std::vector<T> read_bin(const std::string &path, size_t count)
{
    std::vector<T> v(count);
    std::ifstream f(path, std::ios::binary);
    if (count && !f.read(reinterpret_cast<char *>(v.data()), count * sizeof(T))) {
        std::fprintf(stderr, "cannot read %s\n", path.c_str());
        std::exit(2);
    }
    return v;
}

void check(cfd_ctx_t *ctx, cfd_status_t s, const char *what)
{
    if (s != CFD_OK) {
        std::fprintf(stderr, "%s: %s (%s)\n", what, cfd_status_string(s), ctx ? cfd_last_error(ctx) : "");
        std::exit(1);
    }
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc != 3 && argc != 4) {
        std::fprintf(stderr, "usage: host_loop <dir> <steps> [device|host|rk3]\n");
        return 2;
    }
    const std::string dir = argv[1];
    const int steps = std::atoi(argv[2]);
    const std::string mode = argc == 4 ? argv[3] : "device";
    int n_rows, sd_node, viscous, les, n_list[4];
    double mach, reynolds, prandtl, t_inf, eps, dt;
    {
        std::ifstream m(dir + "/meta.txt");
        m >> n_rows >> sd_node >> mach >> reynolds >> prandtl >> t_inf >> eps >> viscous >> les >> dt >> n_list[0]
            >> n_list[1] >> n_list[2] >> n_list[3];
        if (!m) {
            std::fprintf(stderr, "bad meta.txt\n");
            return 2;
        }
    }
    const size_t R = (size_t)n_rows;
    auto grid = read_bin<cfd_grid_t>(dir + "/grid.bin", R);
    auto det = read_bin<double>(dir + "/det.bin", R);
    auto deter = read_bin<cfd_determ_t>(dir + "/deter.bin", R);
    auto metric = read_bin<cfd_metric_t>(dir + "/metric.bin", R);
    auto flow = read_bin<cfd_flow_t>(dir + "/flow.bin", R);
    const char *names[4] = {"outlet", "inlet", "boundary", "wall"};
    std::vector<int32_t> lists[4];
    for (int t = 0; t < 4; ++t) lists[t] = read_bin<int32_t>(dir + "/" + names[t] + ".bin", n_list[t]);

    cfd_ctx_t *ctx = nullptr;
    check(nullptr, cfd_ctx_create(&ctx, 0), "cfd_ctx_create");
    check(ctx, cfd_ctx_set_rows(ctx, n_rows), "cfd_ctx_set_rows");
    cfd_params_t prm;
    cfd_params_default(&prm);
    prm.mach = mach;
    prm.reynolds = reynolds;
    prm.prandtl = prandtl;
    prm.t_inf = t_inf;
    prm.weno_eps = eps;
    prm.viscous = viscous;
    prm.les = les;

    cfd_bc_t *bc = nullptr;
    const bool boundary = n_list[0] + n_list[1] + n_list[2] + n_list[3] > 0;
    if (boundary)
        check(ctx, cfd_bc_create(ctx, grid.data(), n_rows, lists[0].data(), n_list[0], lists[1].data(), n_list[1],
                                 lists[2].data(), n_list[2], lists[3].data(), n_list[3], &bc),
              "cfd_bc_create");

    if (mode == "host") {
        // the reference host's vectors, handed over as they are
        std::vector<cfd_column_t> U[3] = {std::vector<cfd_column_t>(R), std::vector<cfd_column_t>(R),
                                          std::vector<cfd_column_t>(R)};
        std::vector<cfd_column_t> Q(R), F(R), E(R), G(R), Fv(R), Ev(R), Gv(R);
        std::vector<cfd_roe_t> roe(R);
        for (int step = 0; step < steps; ++step)
            for (int j = 0; j < 3; ++j) {
                cfd_column_t *Uj = U[j].data();
                check(ctx, cfd_uq(ctx, Uj, Q.data(), grid.data(), det.data(), flow.data(), roe.data(), n_rows),
                      "cfd_uq");
                check(ctx, cfd_viscous(ctx, Uj, F.data(), E.data(), G.data(), Fv.data(), Ev.data(), Gv.data(),
                                       grid.data(), metric.data(), det.data(), flow.data(), n_rows, &prm),
                      "cfd_viscous");
                check(ctx, cfd_weno(ctx, j, mach, dt, deter.data(), det.data(), U[0].data(), U[1].data(), U[2].data(),
                                    grid.data(), Q.data(), metric.data(), roe.data(), Fv.data(), Ev.data(), Gv.data(),
                                    F.data(), E.data(), G.data(), flow.data(), sd_node + 1, &prm, nullptr),
                      "cfd_weno");
                if (bc) check(ctx, cfd_boundary_fill(ctx, bc, flow.data(), mach, 1, sd_node), "cfd_boundary_fill");
            }
    } else {
        // one device buffer per cl::Buffer of Solver.cpp:232-273
        auto alloc = [&](size_t bytes) {
            void *p = nullptr;
            check(ctx, cfd_buffer_alloc(ctx, bytes, &p), "cfd_buffer_alloc");
            return p;
        };
        auto *dGrid = static_cast<cfd_grid_t *>(alloc(R * sizeof(cfd_grid_t)));
        auto *dDet = static_cast<double *>(alloc(R * sizeof(double)));
        auto *dDeter = static_cast<cfd_determ_t *>(alloc(R * sizeof(cfd_determ_t)));
        auto *dMetric = static_cast<cfd_metric_t *>(alloc(R * sizeof(cfd_metric_t)));
        auto *dFlow = static_cast<cfd_flow_t *>(alloc(R * sizeof(cfd_flow_t)));
        auto *dRoe = static_cast<cfd_roe_t *>(alloc(R * sizeof(cfd_roe_t)));
        cfd_column_t *col[10];   // U0 U1 U2 Q F E G Fv Ev Gv
        std::vector<cfd_column_t> zeros(R);
        for (auto &c : col) {
            c = static_cast<cfd_column_t *>(alloc(R * sizeof(cfd_column_t)));
            check(ctx, cfd_buffer_write(ctx, c, zeros.data(), R * sizeof(cfd_column_t)), "zero columns");
        }
        cfd_column_t *U[3] = {col[0], col[1], col[2]}, *Q = col[3], *F = col[4], *E = col[5], *G = col[6],
                     *Fv = col[7], *Ev = col[8], *Gv = col[9];
        check(ctx, cfd_buffer_write(ctx, dGrid, grid.data(), R * sizeof(cfd_grid_t)), "write grid");
        check(ctx, cfd_buffer_write(ctx, dDet, det.data(), R * sizeof(double)), "write det");
        check(ctx, cfd_buffer_write(ctx, dDeter, deter.data(), R * sizeof(cfd_determ_t)), "write deter");
        check(ctx, cfd_buffer_write(ctx, dMetric, metric.data(), R * sizeof(cfd_metric_t)), "write metric");
        check(ctx, cfd_buffer_write(ctx, dFlow, flow.data(), R * sizeof(cfd_flow_t)), "write flow");
        if (mode == "rk3") {
            check(ctx, cfd_rk3_step(ctx, mach, dt, dDeter, dDet, U[0], U[1], U[2], dGrid, Q, dMetric, dRoe, Fv, Ev, Gv,
                                    F, E, G, dFlow, n_rows - 1, sd_node, &prm, bc, steps),
                  "cfd_rk3_step");
        } else {
            for (int step = 0; step < steps; ++step)
                for (int j = 0; j < 3; ++j) {   // j passed per stage
                    cfd_column_t *Uj = U[j];
                    check(ctx, cfd_uq(ctx, Uj, Q, dGrid, dDet, dFlow, dRoe, n_rows), "cfd_uq");
                    check(ctx, cfd_viscous(ctx, Uj, F, E, G, Fv, Ev, Gv, dGrid, dMetric, dDet, dFlow, n_rows, &prm),
                          "cfd_viscous");
                    check(ctx, cfd_weno(ctx, j, mach, dt, dDeter, dDet, U[0], U[1], U[2], dGrid, Q, dMetric, dRoe, Fv,
                                        Ev, Gv, F, E, G, dFlow, sd_node + 1, &prm, nullptr),
                          "cfd_weno");
                    if (bc) check(ctx, cfd_boundary_fill(ctx, bc, dFlow, mach, 1, sd_node), "cfd_boundary_fill");
                }
        }
        check(ctx, cfd_buffer_read(ctx, flow.data(), dFlow, R * sizeof(cfd_flow_t)), "read flow");
    }
    std::ofstream out(dir + "/flow_out.bin", std::ios::binary);
    out.write(reinterpret_cast<const char *>(flow.data()), R * sizeof(cfd_flow_t));
    if (bc) cfd_bc_destroy(bc);
    cfd_ctx_destroy(ctx);
    std::printf("host_loop: %d steps on %d rows (%s)\n", steps, n_rows, mode.c_str());
    return 0;
}
