// ref_driver.cpp - runs the reference's own class XFLUIDS / class Fluid (compiled from the
// unmodified reference sources against the project's serial SYCL host shim) on a given state and
// dumps the raw FP64 arrays after every RK stage. Used only to pin the oracle (test infrastructure).
//
// Environment:
//   XFREF_IN     input file: int32 E, int64 ncell, int32 hasT, E*ncell doubles U (AoS), [ncell doubles T]
//   XFREF_OUT    output file: per stage record int32 step, int32 flag, double dt, double t, then
//                U, U1, LU (E*ncell each), rho, p, u, v, w, c, H, T (ncell each), y (NUM_SPECIES*ncell)
//   XFREF_STEPS  number of time steps
//   XFREF_TEND   end time (the dt clip of XFLUIDS::Evolution)
//   XFREF_TIMING if set: no per-stage records; the time-step loop is timed (steady clock) and one
//                line "xfref_time <seconds> <steps>" is printed, the output file gets the final U
//   XFREF_TRANSPORT (viscous builds) file for the fitted transport coefficients of Setup: int32 NS,
//                int32 order, visc (NS*order), therm (NS*order), Dkj (NS*NS*order), species_chara
//                (NS*SPCH_Sz), Yil_limiter, Dim_limiter (doubles)
// The sequence mirrors main.cpp:36-49 and the loop body of XFLUIDS::Evolution (src/XFLUIDS.cpp:172-214).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "global_class.h"

static void put(FILE *f, const void *p, size_t n) {
    if (fwrite(p, 1, n, f) != n) {
        perror("write");
        exit(3);
    }
}

int main(int argc, char *argv[]) {
    const char *in = getenv("XFREF_IN"), *out = getenv("XFREF_OUT");
    const int nsteps = getenv("XFREF_STEPS") ? atoi(getenv("XFREF_STEPS")) : 1;
    const double tend = getenv("XFREF_TEND") ? atof(getenv("XFREF_TEND")) : 1e300;
    if (!in || !out) {
        fprintf(stderr, "XFREF_IN / XFREF_OUT not set\n");
        return 2;
    }
    Setup setup(argc, argv);
    XFLUIDS solver(setup);
    solver.AllocateMemory(setup.q);
    solver.InitialCondition(setup.q);
    Fluid *fl = solver.fluids[0];
#if Visc
    if (const char *tp = getenv("XFREF_TRANSPORT")) {
        FILE *ft = fopen(tp, "wb");
        const int ns = NUM_SPECIES, order = order_polynominal_fitted;
        put(ft, &ns, 4), put(ft, &order, 4);
        for (int k = 0; k < ns; k++) put(ft, setup.h_thermal.fitted_coefficients_visc[k], 8 * order);
        for (int k = 0; k < ns; k++) put(ft, setup.h_thermal.fitted_coefficients_therm[k], 8 * order);
        for (int k = 0; k < ns * ns; k++) put(ft, setup.h_thermal.Dkj_matrix[k], 8 * order);
        put(ft, setup.h_thermal.species_chara, 8 * ns * SPCH_Sz);
        put(ft, &setup.BlSz.Yil_limiter, 8), put(ft, &setup.BlSz.Dim_limiter, 8);
        fclose(ft);
    }
#endif
    const size_t ncell = (size_t)setup.BlSz.Xmax * setup.BlSz.Ymax * setup.BlSz.Zmax;

    FILE *fi = fopen(in, "rb");
    int E = 0, hasT = 0;
    long long nc = 0;
    if (!fi || fread(&E, 4, 1, fi) != 1 || fread(&nc, 8, 1, fi) != 1 || fread(&hasT, 4, 1, fi) != 1) {
        fprintf(stderr, "bad input\n");
        return 2;
    }
    if (E != Emax || (size_t)nc != ncell) {
        fprintf(stderr, "input shape mismatch: E %d vs %d, ncell %lld vs %zu\n", E, Emax, nc, ncell);
        return 2;
    }
    if (fread(fl->d_U, sizeof(real_t), E * ncell, fi) != E * ncell) return 2;
    std::memcpy(fl->d_U1, fl->d_U, sizeof(real_t) * E * ncell);
    if (hasT && fread(fl->d_fstate.T, sizeof(real_t), ncell, fi) != ncell) return 2;
    fclose(fi);

    FILE *fo = fopen(out, "wb");
    const bool timing = getenv("XFREF_TIMING") != nullptr;
    solver.physicalTime = 0.0;
    solver.BoundaryCondition(setup.q);
    solver.UpdateStates(setup.q);
    const auto clock0 = std::chrono::steady_clock::now();
    int done = 0;
    for (int step = 1; step <= nsteps && solver.physicalTime < tend; step++) {
        Setup::adv_nd[0].resize(1);
        Setup::sbm_id = 0, Setup::adv_id = 0, Setup::adv_push = true;
        real_t dt = solver.ComputeTimeStep(setup.q);
        if (solver.physicalTime + dt > tend) dt = tend - solver.physicalTime;
        solver.dt = dt;
        const real_t t0 = solver.physicalTime;
        solver.physicalTime += dt;
        for (int flag = 1; flag <= 3; flag++) {
            if (solver.RungeKuttaSP3rd(setup.q, 0, step, t0, flag)) {
                fprintf(stderr, "reference captured an error at step %d stage %d\n", step, flag);
                fclose(fo);
                return 4;
            }
            if (timing) continue;
            double tt = solver.physicalTime;
            put(fo, &step, 4), put(fo, &flag, 4), put(fo, &dt, 8), put(fo, &tt, 8);
            put(fo, fl->d_U, sizeof(real_t) * E * ncell);
            put(fo, fl->d_U1, sizeof(real_t) * E * ncell);
            put(fo, fl->d_LU, sizeof(real_t) * E * ncell);
            FlowData &d = fl->d_fstate;
            real_t *prim[] = {d.rho, d.p, d.u, d.v, d.w, d.c, d.H, d.T};
            for (real_t *a : prim) put(fo, a, sizeof(real_t) * ncell);
            put(fo, d.y, sizeof(real_t) * NUM_SPECIES * ncell);
        }
        done = step;
    }
    if (timing) {
        const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - clock0).count();
        printf("xfref_time %.6f %d\n", sec, done);
        put(fo, fl->d_U, sizeof(real_t) * Emax * ncell);
    }
    fclose(fo);
    return 0;
}
