// xfo_capi.cpp - C interface of the CPU oracle (test infrastructure; see xfo_core.hpp).
//
// Build: g++ -O2 -std=c++17 -fopenmp -ffp-contract=off -fPIC -shared xfo_capi.cpp -o libxfo.so
// -ffp-contract=off keeps a*b+c as two rounded operations on every host (aarch64 would otherwise
// fuse them), which is how the reference CPU build evaluates them on x86-64.
#include <omp.h>

#include <cstdio>
#include <cstring>
#include <new>

#include "xfo_core.hpp"
#include "xfo_count.hpp"

namespace xfo {
thread_local uint64_t Cnt::flops = 0;

template <class R>
struct Solver {
    Config cf;
    Fields<R> f;
    double t = 0.0;

    std::vector<R> &stage_U(int flag) { return flag == 0 ? f.U : f.U1; }

    // XFLUIDS::RungeKuttaSP3rd (src/XFLUIDS.cpp:441-525) without the NaN check.
    void rk_stage(int flag, R dt) {
        std::vector<R> &UI = flag == 1 ? f.U : f.U1;
        boundary(cf, UI.data());
        update_states(cf, f, UI);
        compute_lu(cf, f, UI);
        update_rk3(cf, f, flag, dt);
    }
};

template <class R>
static void load(Solver<R> &s, const double *U, const double *T) {
    const size_t n = s.cf.ncell(), E = s.cf.E();
    for (size_t q = 0; q < n * E; q++) s.f.U[q] = R(U[q]), s.f.U1[q] = R(U[q]);
    if (T)
        for (size_t q = 0; q < n; q++) s.f.T[q] = R(T[q]);
}
}  // namespace xfo

using namespace xfo;

struct xfo_handle {
    Solver<double> s;
};

extern "C" {

int xfo_set_threads(int n) {
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
}

xfo_handle *xfo_create(const xfg_block *bl, const xfg_scheme *sc, const xfg_thermal *th) {
    xfo_handle *h = new (std::nothrow) xfo_handle();
    if (!h) return nullptr;
    h->s.cf.bl = *bl;
    h->s.cf.sc = *sc;
    h->s.cf.th = *th;
    h->s.f.alloc(h->s.cf);
    return h;
}

void xfo_destroy(xfo_handle *h) { delete h; }

int xfo_set_transport(xfo_handle *h, const xfg_transport *tr) {
    h->s.cf.tr = *tr;
    return 0;
}

int xfo_set_state(xfo_handle *h, const double *U, const double *T) {
    load(h->s, U, T);
    return 0;
}

int xfo_boundary(xfo_handle *h, int flag) {
    boundary(h->s.cf, h->s.stage_U(flag).data());
    return 0;
}

int xfo_update_states(xfo_handle *h, int flag) {
    update_states(h->s.cf, h->s.f, h->s.stage_U(flag));
    return 0;
}

int xfo_compute_lu(xfo_handle *h, int flag) {
    compute_lu(h->s.cf, h->s.f, h->s.stage_U(flag));
    return 0;
}

int xfo_update_rk3(xfo_handle *h, int flag, double dt) {
    update_rk3(h->s.cf, h->s.f, flag, dt);
    return 0;
}

int xfo_get_dt(xfo_handle *h, double *dt) {
    *dt = get_dt(h->s.cf, h->s.f);
    return 0;
}

// One step of XFLUIDS::Evolution (src/XFLUIDS.cpp:196-214): dt from the current primitives,
// clipped to target_t, then the three RK stages.
int xfo_step(xfo_handle *h, double target_t, double *t, double *dt_out) {
    double dt = get_dt(h->s.cf, h->s.f);
    if (h->s.t + dt > target_t) dt = target_t - h->s.t;
    h->s.t += dt;
    for (int flag = 1; flag <= 3; flag++) h->s.rk_stage(flag, dt);
    if (t) *t = h->s.t;
    if (dt_out) *dt_out = dt;
    return 0;
}

int xfo_set_time(xfo_handle *h, double t) {
    h->s.t = t;
    return 0;
}

// Copy an array out in the reference layout; ids follow enum xfg_array.
int xfo_get_array(xfo_handle *h, int which, double *out) {
    Fields<double> &f = h->s.f;
    const std::vector<double> *src = nullptr;
    switch (which) {
    case XFG_U: src = &f.U; break;
    case XFG_U1: src = &f.U1; break;
    case XFG_LU: src = &f.LU; break;
    case XFG_RHO: src = &f.rho; break;
    case XFG_P: src = &f.p; break;
    case XFG_U_VEL: src = &f.u; break;
    case XFG_V_VEL: src = &f.v; break;
    case XFG_W_VEL: src = &f.w; break;
    case XFG_C: src = &f.c; break;
    case XFG_H: src = &f.H; break;
    case XFG_T: src = &f.T; break;
    case XFG_GAMMA: src = &f.gamma; break;
    case XFG_E: src = &f.e; break;
    case XFG_CP: src = &f.Cp; break;
    case XFG_R: src = &f.Rm; break;
    case XFG_Y: src = &f.y; break;
    case XFG_FWX: src = &f.Fw[0]; break;
    case XFG_FWY: src = &f.Fw[1]; break;
    case XFG_FWZ: src = &f.Fw[2]; break;
    default: return -1;
    }
    std::memcpy(out, src->data(), src->size() * sizeof(double));
    return 0;
}

// Algorithmic flop count of nsteps steps (after the initial UpdateStates) on the given state,
// single-threaded with the counting scalar. counts[0..8]: boundary, update_states, local eigen +
// GLF maxima, faces x, faces y, faces z, divergence, RK update, dt. Returns 0.
int xfo_count_flops(const xfg_block *bl, const xfg_scheme *sc, const xfg_thermal *th, const double *U,
                    const double *T, int nsteps, uint64_t *counts) {
    int saved = omp_get_max_threads();
    omp_set_num_threads(1);
    Solver<Cnt> s;
    s.cf.bl = *bl;
    s.cf.sc = *sc;
    s.cf.th = *th;
    s.f.alloc(s.cf);
    load(s, U, T);
    for (int q = 0; q < 9; q++) counts[q] = 0;
    boundary(s.cf, s.f.U.data());
    update_states(s.cf, s.f, s.f.U);
    const int dims[3] = {bl->DimX, bl->DimY, bl->DimZ};
    for (int step = 0; step < nsteps; step++) {
        Cnt::flops = 0;
        Cnt dt = get_dt(s.cf, s.f);
        counts[8] += Cnt::flops;
        for (int flag = 1; flag <= 3; flag++) {
            std::vector<Cnt> &UI = flag == 1 ? s.f.U : s.f.U1;
            Cnt::flops = 0;
            boundary(s.cf, UI.data());
            counts[0] += Cnt::flops, Cnt::flops = 0;
            update_states(s.cf, s.f, UI);
            counts[1] += Cnt::flops, Cnt::flops = 0;
            lu_eigen(s.cf, s.f);
            counts[2] += Cnt::flops, Cnt::flops = 0;
            for (int d = 0; d < 3; d++) {
                if (!dims[d]) continue;
                lu_faces(s.cf, s.f, UI, d);
                counts[3 + d] += Cnt::flops, Cnt::flops = 0;
            }
            lu_divergence(s.cf, s.f);
            counts[6] += Cnt::flops, Cnt::flops = 0;
            update_rk3(s.cf, s.f, flag, dt);
            counts[7] += Cnt::flops, Cnt::flops = 0;
        }
    }
    omp_set_num_threads(saved);
    return 0;
}

}  // extern "C"
