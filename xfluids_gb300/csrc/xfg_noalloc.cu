// xfg_noalloc.cu - the convective right-hand side of one state without any device allocation.
//
// Some callers cannot call cudaMalloc: plugins loaded into a host application that owns every
// device allocation (its own pool allocator, a fixed memory budget), and real-time or
// latency-bound loops in which an allocation, and the synchronisation the driver allocator may
// imply, is not allowed. xfg_compute_lu_noalloc serves them: the caller passes device pointers to
// the input state and to the output right-hand side, and every intermediate array (primitives,
// physical fluxes, face fluxes, the SoA copy of the state) lives in one file-scope __device__
// array of fixed size, g_noalloc_scratch, which every GPU that loads the library holds until the
// process exits. The first call on a device looks up the array's device address with that device
// current; make that first call before any stream capture.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/xfluids_gb300.h"
#define XFG_KNS noalloc
#include "xfg_kernels.cuh"
#include "xfg_ops.h"

namespace {

// 64 MiB of scratch: 8 Mi doubles.
constexpr size_t kScratchDoubles = (size_t)XFG_NOALLOC_MAX_SCRATCH_BYTES / sizeof(double);
__device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::once_flag g_once[kMaxDevices];
double *g_scratch_ptr[kMaxDevices];
cudaError_t g_setup_err[kMaxDevices];

int fail(int code, const char *msg, cudaError_t e = cudaSuccess) {
    char buf[512];
    if (e != cudaSuccess)
        snprintf(buf, sizeof buf, "xfg_compute_lu_noalloc: %s: %s", msg, cudaGetErrorString(e));
    else
        snprintf(buf, sizeof buf, "xfg_compute_lu_noalloc: %s", msg);
    xfg::set_last_error(buf);  // read back with xfg_last_error()
    return code;
}

// Device address of the scratch array on the current device; the first call on a device looks it
// up (cudaGetSymbolAddress), later calls reuse it.
double *scratch_for(int dev, cudaError_t *err) {
    std::call_once(g_once[dev], [dev] {
        double *p = nullptr;
        g_setup_err[dev] = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
        g_scratch_ptr[dev] = g_setup_err[dev] == cudaSuccess ? p : nullptr;
    });
    *err = g_setup_err[dev];
    return g_scratch_ptr[dev];
}

__global__ void k_aos_to_soa_na(const double *__restrict__ aos, double *__restrict__ soa, int E, long long N,
                                long long P) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * E) return;
    soa[(t % E) * P + t / E] = aos[t];
}
__global__ void k_soa_to_aos_na(const double *__restrict__ soa, double *__restrict__ aos, int E, long long N,
                                long long P) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * E) return;
    aos[t] = soa[(t % E) * P + t / E];
}

size_t up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace

extern "C" int xfg_compute_lu_noalloc(const xfg_block *block, const xfg_scheme *scheme, const xfg_thermal *thermal,
                                      const double *U_aos, const double *T, double *LU_aos, void *stream) {
    if (!block || !scheme || !thermal || !U_aos || !LU_aos) return fail(-1, "null argument");
    // the checks of xfg_create first (scheme switches, sizes, the face launches' grid limits), so
    // that nothing is launched for a block the kernels cannot cover
    if (xfg::validate_block_scheme(block, scheme, thermal)) return -1;
    if (scheme->precision != XFG_FP64 && scheme->precision != XFG_FP64_STRICT)
        return fail(-1, "xfg_compute_lu_noalloc serves the FP64 forms (precision 0 or 2)");
    if (scheme->viscous) return fail(-1, "xfg_compute_lu_noalloc has no viscous fluxes (they need transport data)");
    if (scheme->positivity)
        return fail(-1, "xfg_compute_lu_noalloc has no positivity limiter (it needs the step's GetDt maxima)");
    if (scheme->cop && !T) return fail(-1, "a mixture needs the temperature T (Newton warm start)");
    const xfg::Ops *ops = xfg::find_ops(scheme->cop ? 1 : 0, scheme->cop ? scheme->num_species : 1,
                                        scheme->scheme_order, scheme->precision);
    if (!ops) return fail(-1, "no kernels built for this scheme");
    const int dims[3] = {block->DimX, block->DimY, block->DimZ};
    const int ndim = dims[0] + dims[1] + dims[2];
    const int E = scheme->cop ? scheme->num_species + 4 : 5, NS = scheme->cop ? scheme->num_species : 1;
    const long long N = (long long)block->Xmax * block->Ymax * block->Zmax;
    const long long P = (long long)up((size_t)N, 64);
    // U, LU, 12 primitives, y and the per-cell sound-speed terms of a mixture (3 + NS - 1), F and
    // Fw per active direction, and for the single-gas FP64 fast kernels sqrt(rho), 1/sqrt(rho) and
    // 3 |lambda| per direction; 1024 doubles of small words
    const bool fast1 = !scheme->cop && scheme->precision == XFG_FP64;
    const size_t arrays =
        2 * E + 12 + (scheme->cop ? NS + 3 + (NS - 1) : 0) + 2 * E * ndim + (fast1 ? 2 + 3 * ndim : 0);
    const size_t need_doubles = arrays * (size_t)P + 1024;
    if (need_doubles > kScratchDoubles)
        return fail(-2, "block too large for the fixed scratch of xfg_compute_lu_noalloc "
                        "(needs more than XFG_NOALLOC_MAX_SCRATCH_BYTES)");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(-3, "cudaGetDevice failed", e);
    if (dev < 0 || dev >= kMaxDevices) return fail(-3, "device ordinal out of range");
    double *base = scratch_for(dev, &e);
    if (!base) return fail(-3, "cudaGetSymbolAddress of the scratch array failed", e);
    cudaStream_t st = (cudaStream_t)stream;

    xfg::LaunchCtx c;
    std::memset(&c, 0, sizeof c);
    double *p = base;
    auto take = [&](int comps) { double *r = p; p += (size_t)comps * P; return r; };
    xfg::DevFields &f = c.f;
    f.U = take(E);
    f.U1 = f.U;  // no RK stage here
    f.LU = take(E);
    f.rho = take(1), f.u = take(1), f.v = take(1), f.w = take(1), f.p = take(1), f.H = take(1);
    f.c = take(1), f.T = take(1), f.gamma = take(1), f.e = take(1), f.Cp = take(1), f.R = take(1);
    if (scheme->cop) f.y = take(NS), f.xc = take(3 + (NS - 1));
    for (int d = 0; d < 3; d++)
        if (dims[d]) f.F[d] = take(E), f.Fw[d] = take(E);
    if (fast1) {
        f.sr = take(1), f.isr = take(1);
        for (int d = 0; d < 3; d++)
            if (dims[d]) f.eab[d] = take(3);
    }
    unsigned long long *small = (unsigned long long *)p;  // 1024 doubles of small words
    f.lam = small;
    unsigned long long *glf = small + 8;
    f.dtbuf = nullptr;
    f.err = (int *)(small + 32);
    c.g.Xmax = block->Xmax, c.g.Ymax = block->Ymax, c.g.Zmax = block->Zmax;
    c.g.Xi = block->X_inner, c.g.Yi = block->Y_inner, c.g.Zi = block->Z_inner;
    c.g.Bx = block->Bwidth_X, c.g.By = block->Bwidth_Y, c.g.Bz = block->Bwidth_Z;
    c.g.dimx = block->DimX, c.g.dimy = block->DimY, c.g.dimz = block->DimZ;
    c.g._dx = block->_dx, c.g._dy = block->_dy, c.g._dz = block->_dz;
    geo_split_spacing(c.g);
    c.g.dx = block->dx, c.g.dy = block->dy, c.g.dz = block->dz;
    c.g.pitch = P;
    for (int n = 0; n < XFG_MAX_SPECIES; n++) c.th.Ri[n] = thermal->Ri[n], c.th._Wi[n] = thermal->_Wi[n];
    for (int q = 0; q < XFG_MAX_SPECIES * 21; q++) c.th.Hia[q] = thermal->Hia[q];
    for (int q = 0; q < XFG_MAX_SPECIES * 6; q++) c.th.Hib[q] = thermal->Hib[q];
    c.th.nasa = scheme->thermo ? 1 : 0;
    c.th.ncop_gamma = scheme->ncop_gamma;
    c.st = st;
    c.artificial = scheme->artificial_type;
    c.ghost = scheme->ghost_species;
    for (int q = 0; q < 6; q++) c.bc[q] = block->Boundarys[q];
    c.glf = scheme->artificial_type == XFG_GLF ? (const double *)glf : nullptr;
    c.precision = scheme->precision;

    // the scratch keeps the previous call's contents: clear the words that must start at zero
    // (dt maxima, GLF maxima of this state only, error words)
    e = cudaMemsetAsync(small, 0, 1024 * sizeof(double), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(f.LU, 0, (size_t)E * P * sizeof(double), st);  // ghost cells of LU
    if (e != cudaSuccess) return fail(-3, "cudaMemsetAsync failed", e);
    const long long tot = N * E;
    k_aos_to_soa_na<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(U_aos, f.U, E, N, P);
    if (T) {
        e = cudaMemcpyAsync(f.T, T, (size_t)N * sizeof(double), cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return fail(-3, "cudaMemcpyAsync of T failed", e);
    }
    ops->bc(c, f.U, nullptr);
    ops->states(c, f.U, 0, 0);
    if (scheme->artificial_type == XFG_GLF) ops->glf(c, glf, 0);
    for (int d = 0; d < 3; d++)
        if (dims[d]) ops->faces(c, d, f.U, 0);
    ops->div_rk(c, 0, 0.0, nullptr, 0, 1, 0);
    k_soa_to_aos_na<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(f.LU, LU_aos, E, N, P);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(-3, "kernel launch failed", e);
    return 0;
}
