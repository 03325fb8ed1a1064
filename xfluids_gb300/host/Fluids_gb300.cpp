// Fluids_gb300.cpp - drop-in replacement of the reference's src/Fluids.cpp: class Fluid
// (src/global_class.h:14-55) implemented over the C ABI of libxfluids_gb300 (include/xfluids_gb300.h).
//
// Build it in place of src/Fluids.cpp, link -lxfluids_gb300 -lcudart; XFLUIDS.cpp, main.cpp and
// read_ini/* stay unchanged. The reference-visible buffers (d_U, d_U1, d_LU, Ubak, h_*, d_fstate)
// keep their layouts and are allocated through the reference's queue as before, so output,
// checkpoint and restart code keep working; the CUDA handle holds the state in its own SoA layout:
//   - InitialU runs the sample's initial condition into d_U, then loads d_U (and T) into the handle;
//   - the primitives are mirrored into d_fstate only where XFLUIDS can read them: Output reads them
//     at the top of an iteration (those of the step's third UpdateStates, or of main.cpp's initial
//     one) and after a reported error (those of the failing stage). UpdateFluidStates therefore
//     mirrors on the initial call, on the third stage of a step and when it reports an error, and
//     EstimateFluidNAN mirrors before it reports one; the first two stages' primitives stay in the
//     handle (XFLUIDS::RungeKuttaSP3rd reads none of them, src/XFLUIDS.cpp:441-525);
//   - UpdateFluidURK3 with flag 3 (end of a step) mirrors U back into d_U (CopyToUbak reads it at
//     the top of every iteration, src/XFLUIDS.cpp:174).
// Chemistry (ODESolver), viscosity and the SBI diagnostics are outside the ported path.
#include <cstdio>
#include <cstring>
#include <unordered_map>

#include "global_class.h"
#include "solver_Ini/Ini_block.h"
#include "xfluids_gb300.h"

namespace {
std::unordered_map<const Fluid *, xfg_handle *> g_handles;
// RK stage the next UpdateFluidStates belongs to (1..3), from the last UpdateFluidURK3 flag;
// 0 before the first step (main.cpp's initial UpdateStates)
std::unordered_map<const Fluid *, int> g_next_stage;

xfg_handle *H(const Fluid *f) { return g_handles.at(f); }

void check(int rc, const char *what) {
    if (rc < 0) {
        std::fprintf(stderr, "xfluids_gb300: %s failed (%d): %s\n", what, rc, xfg_last_error());
        std::exit(EXIT_FAILURE);  // the reference's own convention for device errors (compile_sycl.h:67-80)
    }
}

xfg_block to_block(const Setup &s) {
    xfg_block b{};
    const Block &bl = s.BlSz;
    b.Xmax = bl.Xmax, b.Ymax = bl.Ymax, b.Zmax = bl.Zmax;
    b.X_inner = bl.X_inner, b.Y_inner = bl.Y_inner, b.Z_inner = bl.Z_inner;
    b.Bwidth_X = bl.Bwidth_X, b.Bwidth_Y = bl.Bwidth_Y, b.Bwidth_Z = bl.Bwidth_Z;
    b.DimX = bl.DimX, b.DimY = bl.DimY, b.DimZ = bl.DimZ;
    b.dx = bl.dx, b.dy = bl.dy, b.dz = bl.dz, b._dx = bl._dx, b._dy = bl._dy, b._dz = bl._dz;
    b.CFLnumber = bl.CFLnumber;
    for (int q = 0; q < 6; q++) b.Boundarys[q] = (int)s.Boundarys[q];
    return b;
}

xfg_scheme to_scheme() {
    xfg_scheme s{};
#ifdef COP
    s.cop = 1;
#endif
    s.num_species = NUM_SPECIES;
    s.scheme_order = SCHEME_ORDER;
    s.artificial_type = Artificial_type;
    s.thermo = Thermo;
#ifdef GhostSpecies
    s.ghost_species = 1;
#endif
#ifdef NCOP_Gamma
    s.ncop_gamma = NCOP_Gamma;
#else
    s.ncop_gamma = 1.4;
#endif
    s.precision = XFG_FP64;
    s.positivity = PositivityPreserving ? 1 : 0;  // read_json.cpp:68
#if Visc
    s.viscous = 1 | (Visc_Heat ? 2 : 0) | (Visc_Diffu ? 4 : 0);  // cmake/init_options.cmake:81-91
#endif
    return s;
}

#if Visc
// Setup's fitted transport coefficients (src/read_ini/src/viscfit.cpp:148-196, GetFitCoefficient) and the
// diffusion limiters of the block, packed densely with the species count as stride.
xfg_transport to_transport(const Setup &s) {
    xfg_transport t{};
    const int ns = NUM_SPECIES, m = XFG_FIT_ORDER;
    t.num_species = ns;
    for (int k = 0; k < ns; k++)
        for (int i = 0; i < m; i++) {
            t.visc[k * m + i] = s.h_thermal.fitted_coefficients_visc[k][i];
            t.therm[k * m + i] = s.h_thermal.fitted_coefficients_therm[k][i];
        }
    for (int kj = 0; kj < ns * ns; kj++)
        for (int i = 0; i < m; i++) t.dkj[kj * m + i] = s.h_thermal.Dkj_matrix[kj][i];
    for (int q = 0; q < ns * XFG_SPCH; q++) t.species_chara[q] = s.h_thermal.species_chara[q];
    t.yil_limiter = s.BlSz.Yil_limiter, t.dim_limiter = s.BlSz.Dim_limiter;
    return t;
}
#endif

xfg_thermal to_thermal(const Setup &s) {
    xfg_thermal t{};
    t.num_species = NUM_SPECIES;
#ifdef COP
    for (int n = 0; n < NUM_SPECIES; n++) {
        t.Wi[n] = s.h_thermal.Wi[n], t._Wi[n] = s.h_thermal._Wi[n], t.Ri[n] = s.h_thermal.Ri[n];
        for (int q = 0; q < 21; q++) t.Hia[n * 21 + q] = s.h_thermal.Hia[n * 21 + q];
        for (int q = 0; q < 6; q++) t.Hib[n * 6 + q] = s.h_thermal.Hib[n * 6 + q];
    }
#endif
    return t;
}
}  // namespace

Fluid::Fluid(Setup &setup) : Fs(setup), q(setup.q), rank(0), nranks(1), SBIOutIter(0) {
    MPI_BCs_time = 0.0, MPI_trans_time = 0.0, error_patched_times = 0;
}

Fluid::~Fluid() {
    auto it = g_handles.find(this);
    if (it != g_handles.end()) xfg_destroy(it->second), g_handles.erase(it);
    g_next_stage.erase(this);
    for (real_t *p : {d_U, d_U1, d_LU, Ubak, d_FluxF, d_FluxG, d_FluxH, d_wallFluxF, d_wallFluxG, d_wallFluxH})
        if (p) sycl::free(p, q);
}

void Fluid::initialize(int n) {
    Fluid_name = Fluids_name[n];
    material_property.Mtrl_ind = Fs.material_props[n][0];
    material_property.Rgn_ind = Fs.material_props[n][1];
    material_property.Gamma = Fs.material_props[n][2];
}

void Fluid::AllocateFluidMemory(sycl::queue &q) {
    const size_t cells = (size_t)Fs.BlSz.Xmax * Fs.BlSz.Ymax * Fs.BlSz.Zmax;
    const size_t bytes = cells * sizeof(real_t), cellbytes = Emax * bytes;
    h_U = static_cast<real_t *>(sycl::malloc_host(cellbytes, q));
    h_U1 = static_cast<real_t *>(sycl::malloc_host(cellbytes, q));
    h_LU = static_cast<real_t *>(sycl::malloc_host(cellbytes, q));
    real_t **hp[] = {&h_fstate.rho, &h_fstate.p, &h_fstate.c, &h_fstate.H, &h_fstate.u, &h_fstate.v,
                     &h_fstate.w, &h_fstate.T, &h_fstate.e, &h_fstate.gamma};
    for (real_t **a : hp) *a = static_cast<real_t *>(sycl::malloc_host(bytes, q));
    h_fstate.y = static_cast<real_t *>(sycl::malloc_host(bytes * NUM_SPECIES, q));
    d_U = static_cast<real_t *>(sycl::malloc_device(cellbytes, q));
    d_U1 = static_cast<real_t *>(sycl::malloc_device(cellbytes, q));
    d_LU = static_cast<real_t *>(sycl::malloc_device(cellbytes, q));
    Ubak = static_cast<real_t *>(sycl::malloc_shared(cellbytes, q));
    // arrays the sample initial conditions (InitialUFKernel) write
    for (real_t **a : {&d_FluxF, &d_FluxG, &d_FluxH, &d_wallFluxF, &d_wallFluxG, &d_wallFluxH})
        *a = static_cast<real_t *>(sycl::malloc_device(cellbytes, q));
    real_t **dp[] = {&d_fstate.rho, &d_fstate.p, &d_fstate.c, &d_fstate.u, &d_fstate.v, &d_fstate.w, &d_fstate.e,
                     &d_fstate.T, &d_fstate.H, &d_fstate.Ri, &d_fstate.Cp, &d_fstate.gamma};
    for (real_t **a : dp) *a = static_cast<real_t *>(sycl::malloc_device(bytes, q));
    d_fstate.y = static_cast<real_t *>(sycl::malloc_device(bytes * NUM_SPECIES, q));
    d_fstate.hi = static_cast<real_t *>(sycl::malloc_device(bytes * NUM_SPECIES, q));
    q.memset(d_fstate.T, 0, bytes).wait();
    MemMbSize = double(cellbytes >> 20) * 4.0, MPIMbSize = 0.0;

    xfg_block b = to_block(Fs);
    xfg_scheme s = to_scheme();
    xfg_thermal t = to_thermal(Fs);
    xfg_handle *h = nullptr;
    check(xfg_create(&b, &s, &t, Fs.DeviceSelect.size() > 2 ? Fs.DeviceSelect[2] : 0, &h), "xfg_create");
    g_handles[this] = h;
#if Visc
    xfg_transport tr = to_transport(Fs);
    check(xfg_set_transport(h, &tr), "xfg_set_transport");
#endif
}

void Fluid::InitialU(sycl::queue &q) {
    InitializeFluidStates(q, Fs.BlSz, Fs.ini, material_property, Fs.d_thermal, d_fstate, d_U, d_U1, d_LU, d_FluxF,
                          d_FluxG, d_FluxH, d_wallFluxF, d_wallFluxG, d_wallFluxH);
    q.wait();
    check(xfg_set_state(H(this), d_U, d_fstate.T), "xfg_set_state");
    g_next_stage[this] = 0;
}

void Fluid::BoundaryCondition(sycl::queue &q, BConditions BCs[6], int flag) {
    check(xfg_boundary(H(this), flag), "xfg_boundary");
}

// The primitives of the handle's last UpdateFluidStates into the reference-visible d_fstate arrays
// that XFLUIDS::Output / CopyDataFromDevice read (src/XFLUIDS.cpp:726-760).
static void mirror_primitives(xfg_handle *h, FlowData &d) {
    const int ids[] = {XFG_RHO, XFG_P, XFG_U_VEL, XFG_V_VEL, XFG_W_VEL, XFG_C, XFG_H, XFG_T, XFG_GAMMA, XFG_E};
    real_t *dst[] = {d.rho, d.p, d.u, d.v, d.w, d.c, d.H, d.T, d.gamma, d.e};
    for (int n = 0; n < 10; n++) check(xfg_get_array(h, ids[n], dst[n]), "xfg_get_array");
#ifdef COP
    check(xfg_get_array(h, XFG_Y, d.y), "xfg_get_array");
#endif
}

std::pair<bool, std::vector<float>> Fluid::UpdateFluidStates(sycl::queue &q, int flag) {
    int err = 0;
    std::vector<float> timers(4, 0.f);
    check(xfg_update_states(H(this), flag, &err, timers.data()), "xfg_update_states");
    const int stage = g_next_stage[this];
    if (err || stage == 0 || stage == 3) mirror_primitives(H(this), d_fstate);
    return std::make_pair(err != 0, timers);
}

std::vector<float> Fluid::ComputeFluidLU(sycl::queue &q, int flag) {
    std::vector<float> timers(23, 0.f);
    check(xfg_compute_lu(H(this), flag, timers.data()), "xfg_compute_lu");
    return timers;
}

void Fluid::UpdateFluidURK3(sycl::queue &q, int flag, real_t const dt) {
    check(xfg_update_rk3(H(this), flag, dt), "xfg_update_rk3");
    g_next_stage[this] = flag % 3 + 1;
    if (flag == 3) check(xfg_get_array(H(this), XFG_U, d_U), "xfg_get_array");  // CopyToUbak / Output read d_U
}

real_t Fluid::GetFluidDt(sycl::queue &q, const int Iter, const real_t physicalTime) {
    double dt = 0.0;
    check(xfg_get_dt(H(this), &dt), "xfg_get_dt");
    return dt;
}

bool Fluid::EstimateFluidNAN(sycl::queue &q, int flag) {
    int err = 0, pos[XFG_MAX_EQ + 4] = {0};
    int rc = xfg_estimate_nan(H(this), flag, &err, pos);
    check(rc < 0 ? rc : 0, "xfg_estimate_nan");
    if (!err) return false;
    mirror_primitives(H(this), d_fstate);  // the error output reads this stage's primitives
    std::cout << "\nErrors of LU[";
    for (int n = 0; n < Emax - 1; n++) std::cout << pos[n] << ", ";
    std::cout << pos[Emax - 1] << "] located at (i, j, k)= (" << pos[Emax + 1] << ", " << pos[Emax + 2] << ", "
              << pos[Emax + 3] << ") inside the step " << flag << " of RungeKutta captured.\n";
    return true;
}

void Fluid::ODESolver(sycl::queue &q, real_t Time) {
    std::fprintf(stderr, "xfluids_gb300: chemical sources are outside the ported path\n");
    std::exit(EXIT_FAILURE);
}

void Fluid::AllCountsHeader() {}
void Fluid::AllCountsPush(sycl::queue &q, const size_t Iter, const real_t time) {}
void Fluid::GetTheta(sycl::queue &q) {}
