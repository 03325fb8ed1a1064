// dropin_sequence.cpp - the call sequence of the reference's time loop over the C ABI, timed beside
// the graph-replayed fused steps (test program of tests/test_dropin_sequence_gpu.py).
//
// XFLUIDS::Evolution (src/XFLUIDS.cpp:167-214) with the C++ drop-in (xfluids_gb300/host/
// Fluids_gb300.cpp) performs per step: CopyToUbak (a copy of d_U into the managed Ubak, :174 and
// :644-650), ComputeTimeStep -> GetFluidDt, then RungeKuttaSP3rd (:441-525) for flags 1, 2, 3:
// BoundaryCondition, UpdateStates (the drop-in mirrors the primitives into d_fstate on the third
// stage), ComputeLU, EstimateNAN (ESTIM_NAN is on by default, cmake/init_options.cmake:7),
// UpdateU (the drop-in mirrors U into d_U after the third stage). This program issues exactly those
// C ABI calls and copies on the 2D isentropic vortex (periodic [0,10]^2, WENO5 LLF, FP64), times
// them with a steady clock (every call synchronises), and times the same steps through
// xfg_advance on a second handle. Prints one JSON line.
//
//   dropin_sequence N STEPS
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "xfluids_gb300.h"

static void ck(int rc, const char *what) {
    if (rc < 0) {
        std::fprintf(stderr, "%s failed (%d): %s\n", what, rc, xfg_last_error());
        std::exit(2);
    }
}
static void cuck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        std::fprintf(stderr, "%s failed: %s\n", what, cudaGetErrorString(e));
        std::exit(2);
    }
}

int main(int argc, char **argv) {
    const int n = argc > 1 ? std::atoi(argv[1]) : 256, steps = argc > 2 ? std::atoi(argv[2]) : 3;
    const int B = 4;
    xfg_block b{};
    b.X_inner = b.Y_inner = n, b.Z_inner = 1;
    b.Bwidth_X = b.Bwidth_Y = B, b.Bwidth_Z = 0;
    b.Xmax = b.Ymax = n + 2 * B, b.Zmax = 1;
    b.DimX = b.DimY = 1, b.DimZ = 0;
    b.dx = b.dy = 10.0 / n, b.dz = 1.0;
    b._dx = b._dy = 1.0 / b.dx, b._dz = 1.0;
    b.CFLnumber = 0.5;
    for (int q = 0; q < 6; q++) b.Boundarys[q] = XFG_PERIODIC;
    xfg_scheme s{};
    s.num_species = 1, s.scheme_order = 5, s.artificial_type = XFG_LLF, s.thermo = 1, s.ncop_gamma = 1.4;
    s.precision = XFG_FP64;
    xfg_thermal th{};
    th.num_species = 1;

    // the vortex of the reference sample 2D-EulerVortex (ini_sample.hpp:14-89), AoS
    const size_t N = (size_t)b.Xmax * b.Ymax, E = 5;
    std::vector<double> U(N * E);
    const double pi = 3.14159265358979323846, beta = 5.0;
    for (int j = 0; j < b.Ymax; j++)
        for (int i = 0; i < b.Xmax; i++) {
            const double x = (i - B + 0.5) * b.dx - 5.0, y = (j - B + 0.5) * b.dy - 5.0, r2 = x * x + y * y;
            const double rho = std::pow(1.0 - beta * beta * std::exp(1.0 - r2) / 28.0 / pi / pi, 2.5);
            const double k = 0.5 * beta * std::exp(0.5 * (1.0 - r2)) / pi, u = 1.0 - k * y, v = 1.0 + k * x;
            const double p = std::pow(rho, 1.4);
            double *c = &U[E * ((size_t)j * b.Xmax + i)];
            c[0] = rho, c[1] = rho * u, c[2] = rho * v, c[3] = 0.0, c[4] = p / 0.4 + 0.5 * rho * (u * u + v * v);
        }

    // the reference-visible buffers of class Fluid: d_U (AoS), the d_fstate primitives, Ubak (shared)
    double *d_U = nullptr, *Ubak = nullptr, *prim[10];
    cuck(cudaMalloc(&d_U, N * E * 8), "cudaMalloc d_U");
    cuck(cudaMallocManaged(&Ubak, N * E * 8), "cudaMallocManaged Ubak");
    for (auto &a : prim) cuck(cudaMalloc(&a, N * 8), "cudaMalloc d_fstate");
    cuck(cudaMemcpy(d_U, U.data(), N * E * 8, cudaMemcpyHostToDevice), "upload");
    const int pid[10] = {XFG_RHO, XFG_P, XFG_U_VEL, XFG_V_VEL, XFG_W_VEL, XFG_C, XFG_H, XFG_T, XFG_GAMMA, XFG_E};

    xfg_handle *h = nullptr, *g = nullptr;
    ck(xfg_create(&b, &s, &th, 0, &h), "xfg_create");
    ck(xfg_create(&b, &s, &th, 0, &g), "xfg_create");
    auto mirror_prims = [&](xfg_handle *x) {
        for (int q = 0; q < 10; q++) ck(xfg_get_array(x, pid[q], prim[q]), "xfg_get_array");
    };
    auto dropin_steps = [&](int k) {
        for (int st = 0; st < k; st++) {
            cuck(cudaMemcpy(Ubak, d_U, N * E * 8, cudaMemcpyDefault), "CopyToUbak");
            double dt = 0.0;
            ck(xfg_get_dt(h, &dt), "xfg_get_dt");
            for (int flag = 1; flag <= 3; flag++) {
                const int UI = flag == 1 ? 0 : 1;
                int err = 0, pos[XFG_MAX_EQ + 4];
                ck(xfg_boundary(h, UI), "xfg_boundary");
                ck(xfg_update_states(h, UI, &err, nullptr), "xfg_update_states");
                if (flag == 3 || err) mirror_prims(h);
                ck(xfg_compute_lu(h, UI, nullptr), "xfg_compute_lu");
                ck(xfg_estimate_nan(h, flag, &err, pos), "xfg_estimate_nan");
                if (err) {
                    std::fprintf(stderr, "numerical error at step %d stage %d\n", st, flag);
                    std::exit(3);
                }
                ck(xfg_update_rk3(h, flag, dt), "xfg_update_rk3");
                if (flag == 3) ck(xfg_get_array(h, XFG_U, d_U), "xfg_get_array U");
            }
        }
    };
    // InitialU + main.cpp:45-47, one warm-up step, then the same from the initial state, timed
    for (int pass = 0; pass < 2; pass++) {
        cuck(cudaMemcpy(d_U, U.data(), N * E * 8, cudaMemcpyHostToDevice), "upload");
        ck(xfg_set_state(h, d_U, nullptr), "xfg_set_state");
        int err = 0;
        ck(xfg_boundary(h, 0), "xfg_boundary");
        ck(xfg_update_states(h, 0, &err, nullptr), "xfg_update_states");
        mirror_prims(h);
        if (pass == 0) dropin_steps(1);
    }
    ck(xfg_synchronize(h), "sync");
    const auto t0 = std::chrono::steady_clock::now();
    dropin_steps(steps);
    ck(xfg_synchronize(h), "sync");
    const double dropin_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();

    // the same steps as graph-replayed fused steps
    double t = 0.0;
    int done = 0, err = 0;
    float dev_ms = 0.f;
    for (int pass = 0; pass < 2; pass++) {
        ck(xfg_set_state(g, U.data(), nullptr), "xfg_set_state");
        ck(xfg_set_time(g, 0.0), "xfg_set_time");
        ck(xfg_boundary(g, 0), "xfg_boundary");
        ck(xfg_update_states(g, 0, &err, nullptr), "xfg_update_states");
        if (pass == 0) ck(xfg_advance(g, 1, 1e300, &t, &done), "xfg_advance");
    }
    const auto t1 = std::chrono::steady_clock::now();
    ck(xfg_advance_timed(g, steps, 1e300, &t, &done, &dev_ms), "xfg_advance_timed");
    const double adv_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t1).count();

    // the two final states, normwise per component over the inner cells
    std::vector<double> a(N * E), r(N * E);
    ck(xfg_get_array(h, XFG_U, a.data()), "get");
    ck(xfg_get_array(g, XFG_U, r.data()), "get");
    double worst = 0.0;
    for (size_t c = 0; c < E; c++) {
        double num = 0.0, den = 0.0;
        for (int j = B; j < B + n; j++)
            for (int i = B; i < B + n; i++) {
                const size_t q = E * ((size_t)j * b.Xmax + i) + c;
                num = std::fmax(num, std::fabs(a[q] - r[q])), den = std::fmax(den, std::fabs(r[q]));
            }
        worst = std::fmax(worst, den > 0.0 ? num / den : num);
    }
    std::printf("{\"n\": %d, \"steps\": %d, \"dropin_ms_per_step\": %.4f, \"advance_ms_per_step\": %.4f, "
                "\"advance_device_ms_per_step\": %.4f, \"dropin_over_advance\": %.4f, \"max_normwise_diff\": %.3e}\n",
                n, steps, dropin_ms / steps, adv_ms / steps, dev_ms / steps, dropin_ms / adv_ms, worst);
    xfg_destroy(h), xfg_destroy(g);
    cudaFree(d_U), cudaFree(Ubak);
    for (auto p : prim) cudaFree(p);
    return 0;
}
