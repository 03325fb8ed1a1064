// xfg_api.cu - C ABI of the library (include/xfluids_gb300.h): handle, device memory, the
// stage-by-stage entry points that replace class Fluid's methods, the fused step and the
// graph-replayed multi-step advance.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/xfluids_gb300.h"
#define XFG_KNS api
#include "xfg_kernels.cuh"
#include "xfg_ops.h"

using namespace xfg;
using namespace xfg::api;

// ---------------------------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------------------------
static thread_local std::string g_err;
static int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}
#define CK(call)                                                                                       \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) return fail(-2, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                           __FILE__, __LINE__);                                        \
    } while (0)

// ---------------------------------------------------------------------------------------------
// launcher registry
// ---------------------------------------------------------------------------------------------
namespace xfg {
void set_last_error(const char *msg) { g_err = msg; }
static std::vector<const Ops *> &registry() {
    static std::vector<const Ops *> r;
    return r;
}
void register_ops(const Ops *ops) { registry().push_back(ops); }
struct FacesOverride {
    int cop, ns, order, precision;
    FacesFn faces;
};
static std::vector<FacesOverride> &face_overrides() {
    static std::vector<FacesOverride> v;
    return v;
}
void register_faces_override(int cop, int ns, int order, int precision, FacesFn faces) {
    face_overrides().push_back({cop, ns, order, precision, faces});
}
// Tables with their face launcher replaced (built on first use, after every unit registered).
const Ops *find_ops(int cop, int ns, int order, int precision) {
    static std::mutex mu;
    static std::deque<Ops> merged;
    const Ops *base = nullptr;
    for (const Ops *o : registry())
        if (o->cop == cop && o->ns == ns && o->order == order && o->precision == precision) {
            base = o;
            break;
        }
    if (!base) return nullptr;
    for (const FacesOverride &f : face_overrides())
        if (f.cop == cop && f.ns == ns && f.order == order && f.precision == precision) {
            std::lock_guard<std::mutex> lk(mu);
            for (const Ops &m : merged)
                if (m.cop == cop && m.ns == ns && m.order == order && m.precision == precision) return &m;
            merged.push_back(*base);
            merged.back().faces = f.faces;
            return &merged.back();
        }
    return base;
}
}  // namespace xfg

// ---------------------------------------------------------------------------------------------
// helper kernels
// ---------------------------------------------------------------------------------------------
__global__ void k_aos_to_soa(const double *__restrict__ aos, double *__restrict__ soa, int E, long long N,
                             long long P) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * E) return;
    long long id = t / E;
    int n = (int)(t % E);
    soa[n * P + id] = aos[t];
}
__global__ void k_soa_to_aos(const double *__restrict__ soa, double *__restrict__ aos, int E, long long N,
                             long long P) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * E) return;
    long long id = t / E;
    int n = (int)(t % E);
    aos[t] = soa[n * P + id];
}
// FP64 primitive arrays of the single-gas mixed form (which keeps them in FP32 only), filled from
// its FP32 face primitives when a caller reads them: the values of the last UpdateFluidStates.
__global__ void k_prims_from_primf(Geo g, DevFields f, double gamma) {
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= g.ncell()) return;
    const long long P = g.pitch;
    const double rho = f.primf[id], p = f.primf[5 * P + id];
    f.rho[id] = rho, f.u[id] = f.primf[P + id], f.v[id] = f.primf[2 * P + id], f.w[id] = f.primf[3 * P + id];
    f.H[id] = f.primf[4 * P + id], f.p[id] = p, f.c[id] = f.primf[6 * P + id];
    f.gamma[id] = gamma, f.e[id] = p / ((gamma - 1.0) * rho);
}
__global__ void k_set_time(double *dtbuf, double t, double target) {
    dtbuf[0] = 0.0, dtbuf[1] = t, dtbuf[2] = target, dtbuf[3] = 0.0, dtbuf[4] = 0.0;
}

// ---------------------------------------------------------------------------------------------
// handle
// ---------------------------------------------------------------------------------------------
struct xfg_handle {
    int device = 0;
    cudaStream_t st = nullptr;
    xfg_block bl;
    xfg_scheme sc;
    const Ops *ops = nullptr;
    LaunchCtx ctx;
    int E = 5, NS = 1;
    long long N = 0, P = 0;
    void *pool = nullptr;
    size_t pool_bytes = 0;
    double *stage = nullptr;          // AoS staging for transposes
    unsigned long long *glf = nullptr;
    double *host_dtbuf = nullptr;     // pinned mirror of dtbuf
    int *host_err = nullptr;          // pinned mirror of err
    double t = 0.0;
    bool states_ready = false;
    bool transport_ready = false;     // viscous schemes: xfg_set_transport called
    bool fused = false;               // stages run as the fused mixed kernel (xfg_fused.cuh)
    cudaGraphExec_t graph = nullptr;  // one fused step, replayed by xfg_advance
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    alignas(64) CUtensorMap tmap[3];  // fused stages: TMA maps of U, U1, U2 (xfg_fused.cuh)
};

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// TMA maps of the fused stage's state buffers (k_fused_stage_tma): each a 3D tensor (Xmax, Ymax,
// 5 components) of FP64 with row stride Xmax and component stride P cells, copied as boxes of
// FUSED_BOX_X x FUSED_BOX_Y x 5. A map needs 16-byte strides, so Xmax even. The persistent TMA
// kernel is opt-in (XFG_FUSED_TMA=1 in the environment at xfg_create): it computes the same bits as
// the one-tile-per-CTA kernel but measured 6 % slower (its barrier waits outweigh the load latency
// it hides). cuTensorMapEncodeTiled is taken through the runtime's driver entry point, so the
// library links no libcuda.
static bool make_fused_tmaps(xfg_handle *h) {
    const char *env = std::getenv("XFG_FUSED_TMA");
    if (!(env && env[0] == '1') || h->bl.Xmax % 2 || h->bl.DimZ) return false;
    static PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess || q != cudaDriverEntryPointSuccess)
            fn = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }();
    if (!encode) return false;
    const cuuint64_t dim[3] = {(cuuint64_t)h->bl.Xmax, (cuuint64_t)h->bl.Ymax, 5};
    const cuuint64_t stride[2] = {(cuuint64_t)h->bl.Xmax * 8, (cuuint64_t)h->P * 8};
    const cuuint32_t box[3] = {(cuuint32_t)FUSED_BOX_X, (cuuint32_t)FUSED_BOX_Y, 5}, estride[3] = {1, 1, 1};
    double *buf[3] = {h->ctx.f.U, h->ctx.f.U1, h->ctx.f.U2};
    for (int q = 0; q < 3; q++)
        if (encode(&h->tmap[q], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, buf[q], dim, stride, box, estride,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return false;
    return true;
}

// Argument and block checks shared by xfg_create and xfg_compute_lu_noalloc (declared in xfg_ops.h).
namespace xfg {
int validate_block_scheme(const xfg_block *b, const xfg_scheme *s, const xfg_thermal *t) {
    if (!b || !s || !t) return fail(-1, "null argument");
    if (s->scheme_order < 5 || s->scheme_order > 7)
        return fail(-1, "scheme_order must be 5 (WENO5), 6 (WENO-CU6) or 7 (WENO7) (got %d)", s->scheme_order);
    if (s->artificial_type < 1 || s->artificial_type > 3) return fail(-1, "artificial_type must be 1..3");
    if (s->precision < 0 || s->precision > 2) return fail(-1, "precision must be 0 (fp64), 1 (mixed) or 2 (fp64 strict)");
    if (s->positivity != 0 && s->positivity != 1) return fail(-1, "positivity must be 0 or 1");
    if (s->viscous < 0 || s->viscous > 7) return fail(-1, "viscous must be Visc | Visc_Heat << 1 | Visc_Diffu << 2");
    if (s->viscous && !(s->viscous & 1)) return fail(-1, "Visc_Heat / Visc_Diffu need Visc (bit 0)");
    if (s->viscous && !s->cop)
        return fail(-1, "viscous fluxes need a mixture (cop = 1): the single-gas states compute no temperature");
    if (s->cop && (s->num_species < 2 || s->num_species > XFG_MAX_SPECIES))
        return fail(-1, "num_species %d out of range for COP", s->num_species);
    if (!s->cop && s->num_species != 1) return fail(-1, "num_species must be 1 without COP");
    if (s->cop && t->num_species != s->num_species) return fail(-1, "thermal.num_species != scheme.num_species");
    const int dims[3] = {b->DimX, b->DimY, b->DimZ};
    const int inner[3] = {b->X_inner, b->Y_inner, b->Z_inner};
    const int bw[3] = {b->Bwidth_X, b->Bwidth_Y, b->Bwidth_Z};
    const int mx[3] = {b->Xmax, b->Ymax, b->Zmax};
    const int need = s->scheme_order == 7 ? 4 : 3;
    for (int d = 0; d < 3; d++) {
        if (dims[d]) {
            if (bw[d] < need) return fail(-1, "Bwidth of direction %d is %d, the scheme needs >= %d", d, bw[d], need);
            if (inner[d] < bw[d]) return fail(-1, "inner size %d of direction %d below Bwidth %d", inner[d], d, bw[d]);
            if (mx[d] != inner[d] + 2 * bw[d]) return fail(-1, "Xmax/Ymax/Zmax inconsistent in direction %d", d);
        } else if (mx[d] != 1 || inner[d] != 1 || bw[d] != 0) {
            return fail(-1, "absent direction %d must have max = inner = 1 and Bwidth = 0", d);
        }
    }
    if (!(dims[0] || dims[1] || dims[2])) return fail(-1, "no active direction");
    // face launches: 32 x 4 threads per block, grid (x/32, y/4, z) for the x and y sweeps and
    // (x/32, y, z/4) for the z sweep; grid y and z are limited to 65535 blocks
    if (inner[2] + 1 > 65535 || (dims[2] && inner[1] + 1 > 65535) || (inner[1] + 4) / 4 > 65535)
        return fail(-1, "block too elongated for the face launches (Z_inner or, in 3D, Y_inner above 65534)");
    return 0;
}
int pack_transport(const xfg_transport *tr, int ns, std::vector<double> &t, std::vector<float> &tf) {
    if (tr->num_species != ns) return fail(-1, "transport data for %d species, the scheme has %d", tr->num_species, ns);
    t.assign(8 * ns + 2 * ns * ns + ns, 0.0);
    for (int k = 0; k < ns; k++)
        for (int q = 0; q < XFG_FIT_ORDER; q++) {
            t[4 * k + q] = tr->visc[k * XFG_FIT_ORDER + q];
            t[4 * ns + 4 * k + q] = tr->therm[k * XFG_FIT_ORDER + q];
        }
    for (int k = 0; k < ns; k++)
        for (int i = 0; i < ns; i++) {
            const double Wk = tr->species_chara[k * XFG_SPCH + 6], Wi = tr->species_chara[i * XFG_SPCH + 6];
            t[8 * ns + k * ns + i] = std::pow(Wi / Wk, 0.25);
            t[8 * ns + ns * ns + k * ns + i] = std::pow(1.0 + Wk / Wi, -0.5);
        }
    for (int k = 0; k < ns; k++) {
        const double sid = tr->species_chara[k * XFG_SPCH + 8];
        if (!(sid >= 0.0 && sid < ns)) return fail(-1, "species id %g out of range", sid);
        t[8 * ns + 2 * ns * ns + k] = sid;
    }
    tf.assign(8 * ns + 2 * ns * ns, 0.0f);
    for (int k = 0; k < ns; k++) {
        const int ik = (int)t[8 * ns + 2 * ns * ns + k];
        for (int q = 0; q < XFG_FIT_ORDER; q++) {
            tf[4 * k + q] = (float)t[4 * ik + q];
            tf[4 * ns + 4 * k + q] = (float)t[4 * ns + 4 * ik + q];
        }
        for (int i = 0; i < ns; i++) {
            tf[8 * ns + k * ns + i] = (float)t[8 * ns + k * ns + i];
            tf[8 * ns + ns * ns + k * ns + i] = (float)(t[8 * ns + ns * ns + k * ns + i] * 0.5 / std::sqrt(2.0));
        }
    }
    return 0;
}
}  // namespace xfg

extern "C" {

const char *xfg_last_error(void) { return g_err.c_str(); }

const char *xfg_build_info(void) {
    static std::string info;
    if (info.empty()) {
        info = "xfluids_gb300 sm_103a; kernels:";
        for (const Ops *o : registry()) {
            char b[64];
            static const char *pn[3] = {"fp64", "mixed", "fp64strict"};
            snprintf(b, sizeof b, " %s%d/weno%d/%s", o->cop ? "cop" : "ncop", o->ns, o->order, pn[o->precision]);
            info += b;
        }
    }
    return info.c_str();
}

int xfg_create(const xfg_block *block, const xfg_scheme *scheme, const xfg_thermal *thermal, int device,
               xfg_handle **out) {
    if (!out) return fail(-1, "null out");
    *out = nullptr;
    int v = validate_block_scheme(block, scheme, thermal);
    if (v) return v;
    // Mixtures with the positivity limiter keep the no-contraction face sweeps in the FP64 form:
    // the limiter's theta = (rho_low - eps) / (rho_low - rho_high) amplifies the rounding of the
    // high-order flux (contracted faces moved LU by 4e-10 on identical inputs).
    const int table_prec = (scheme->cop && scheme->positivity && scheme->precision == XFG_FP64) ? XFG_FP64_STRICT
                                                                                                : scheme->precision;
    const Ops *ops = find_ops(scheme->cop ? 1 : 0, scheme->cop ? scheme->num_species : 1, scheme->scheme_order,
                              table_prec);
    if (!ops)
        return fail(-1, "no kernels built for cop=%d num_species=%d order=%d precision=%d", scheme->cop,
                    scheme->num_species, scheme->scheme_order, scheme->precision);
    CK(cudaSetDevice(device));
    if (fused_applies(*block, *scheme, ops)) {  // the fused kernels' shared memory, once per device
        const cudaError_t fe = (cudaError_t)ops->fused_prepare();
        if (fe != cudaSuccess) return fail(-2, "fused stage set-up failed: %s", cudaGetErrorString(fe));
    }
    xfg_handle *h = new xfg_handle();
    h->device = device;
    h->bl = *block;
    h->sc = *scheme;
    h->ops = ops;
    h->NS = scheme->cop ? scheme->num_species : 1;
    h->E = scheme->cop ? scheme->num_species + 4 : 5;
    h->N = (long long)block->Xmax * block->Ymax * block->Zmax;
    h->P = (long long)align_up((size_t)h->N, 64);
    const int E = h->E, NS = h->NS;
    const bool mixed = scheme->precision == XFG_MIXED;  // FP32 copies instead of FP64 fluxes
    h->fused = fused_applies(*block, *scheme, ops);
    const int dims[3] = {block->DimX, block->DimY, block->DimZ};
    const size_t arr8 = (size_t)h->P * 8, arr4 = align_up((size_t)h->P * 4, 256);
    // layout of the pool
    size_t nd = 3 * E + 12 + (scheme->cop ? NS : 0);           // U, U1, LU, primitives, y
    if (h->fused) nd += E;                                      // U2, the fused stages' third buffer
    if (scheme->cop && !mixed) nd += 3 + (NS - 1);              // per-cell sound-speed terms
    if (scheme->viscous && !mixed) nd += 9 + 2;                 // velocity derivatives, mu, kappa
    const bool fast1 = !scheme->cop && scheme->precision == XFG_FP64;  // single-gas fast path extras
    if (fast1) nd += 2 + 3 * (block->DimX + block->DimY + block->DimZ);
    const bool mixcop = scheme->cop && mixed;
    for (int d = 0; d < 3; d++)
        if (dims[d] && !mixed) nd += 2 * E;                       // F, Fw
    size_t nf = 0;
    if (mixed) {
        nf = E + 7;
        if (mixcop) nf += NS + 3 + (NS - 1);                     // FP32 y and sound-speed terms
        if (scheme->viscous) nf += 9 + 2 + 1;                    // FP32 derivatives, mu, kappa, T
        for (int d = 0; d < 3; d++)
            if (dims[d]) nf += 2 * E;                             // Ff, Fwf
    }
    const size_t stage_elems = (size_t)h->N * (E > NS ? E : NS);
    // small words; transport tables at +4096 and +6144; scaled thermo table at +8192
    const size_t small = 8192 + align_up(THERMO_SC_BYTES, 256);
    size_t bytes = nd * arr8 + nf * arr4 + align_up(stage_elems * 8, 256) + small;
    cudaError_t e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&h->pool, bytes);
    if (e != cudaSuccess) {
        if (h->st) cudaStreamDestroy(h->st);
        delete h;
        return fail(-3, "device allocation of %.3f GB failed: %s", bytes / 1e9, cudaGetErrorString(e));
    }
    h->pool_bytes = bytes;
    cudaMemsetAsync(h->pool, 0, bytes, h->st);
    char *p = (char *)h->pool;
    auto take8 = [&](size_t count) { double *r = (double *)p; p += count * arr8; return r; };
    auto take4 = [&](size_t count) { float *r = (float *)p; p += count * arr4; return r; };
    DevFields &f = h->ctx.f;
    std::memset(&f, 0, sizeof f);
    f.U = take8(E), f.U1 = take8(E), f.LU = take8(E);
    if (h->fused) f.U2 = take8(E);
    f.rho = take8(1), f.u = take8(1), f.v = take8(1), f.w = take8(1), f.p = take8(1), f.H = take8(1);
    f.c = take8(1), f.T = take8(1), f.gamma = take8(1), f.e = take8(1), f.Cp = take8(1), f.R = take8(1);
    if (scheme->cop) f.y = take8(NS);
    if (scheme->cop && !mixed) f.xc = take8(3 + (NS - 1));
    if (scheme->viscous && !mixed) f.vde = take8(9), f.mu = take8(1), f.kappa = take8(1);
    if (fast1) {
        f.sr = take8(1), f.isr = take8(1);
        for (int d = 0; d < 3; d++)
            if (dims[d]) f.eab[d] = take8(3);
    }
    for (int d = 0; d < 3; d++)
        if (dims[d] && !mixed) f.F[d] = take8(E), f.Fw[d] = take8(E);
    if (mixed) {
        f.Uf = take4(E);
        f.primf = take4(7);
        if (mixcop) f.yf = take4(NS), f.xcf = take4(3 + (NS - 1));
        if (scheme->viscous) f.vdef = take4(9), f.muf = take4(1), f.kappaf = take4(1), f.Tf = take4(1);
        for (int d = 0; d < 3; d++)
            if (dims[d]) f.Ff[d] = take4(E), f.Fwf[d] = take4(E);
    }
    h->stage = (double *)p;
    p += align_up(stage_elems * 8, 256);
    f.lam = (unsigned long long *)p;              // 3 x u64
    h->glf = (unsigned long long *)(p + 64);      // 9 x u64
    f.dtbuf = (double *)(p + 256);                // 8 doubles
    f.err = (int *)(p + 512);                     // 8 ints (+ NaN estimate scratch after)
    if (scheme->viscous) {  // transport tables (xfg_set_transport): FP64 at +4096, FP32 at +6144
        f.tr = (const double *)(p + 4096);
        f.trf = (const float *)(p + 6144);
    }
    // launch context
    Geo &g = h->ctx.g;
    g.Xmax = block->Xmax, g.Ymax = block->Ymax, g.Zmax = block->Zmax;
    g.Xi = block->X_inner, g.Yi = block->Y_inner, g.Zi = block->Z_inner;
    g.Bx = block->Bwidth_X, g.By = block->Bwidth_Y, g.Bz = block->Bwidth_Z;
    g.dimx = block->DimX, g.dimy = block->DimY, g.dimz = block->DimZ;
    g._dx = block->_dx, g._dy = block->_dy, g._dz = block->_dz;
    geo_split_spacing(g);
    g.dx = block->dx, g.dy = block->dy, g.dz = block->dz;
    g.pitch = h->P;
    DevThermo &th = h->ctx.th;
    std::memset(&th, 0, sizeof th);
    for (int n = 0; n < XFG_MAX_SPECIES; n++) th.Ri[n] = thermal->Ri[n], th._Wi[n] = thermal->_Wi[n];
    for (int q = 0; q < XFG_MAX_SPECIES * 21; q++) th.Hia[q] = thermal->Hia[q];
    for (int q = 0; q < XFG_MAX_SPECIES * 6; q++) th.Hib[q] = thermal->Hib[q];
    th.nasa = scheme->thermo ? 1 : 0;
    th.ncop_gamma = scheme->ncop_gamma;
    std::vector<double> hsc(THERMO_SC_DOUBLES);
    std::vector<char> hb(THERMO_SC_BYTES);
    if (scheme->cop) {  // the mixed form's scaled enthalpy tables, FP64 then FP32
        scaled_thermo_table(th, hsc.data());
        std::memcpy(hb.data(), hsc.data(), THERMO_SC_DOUBLES * sizeof(double));
        float *hf = (float *)(hb.data() + THERMO_SC_DOUBLES * sizeof(double));
        for (int q = 0; q < THERMO_SC_DOUBLES; q++) hf[q] = (float)hsc[q];
        double *d = (double *)(p + 8192);
        th.hsc = d;
        th.hscf = (const float *)(d + THERMO_SC_DOUBLES);
        if (cudaMemcpyAsync(d, hb.data(), THERMO_SC_BYTES, cudaMemcpyHostToDevice, h->st) != cudaSuccess) {
            xfg_destroy(h);
            return fail(-2, "upload of the thermo tables failed");
        }
    }
    h->ctx.st = h->st;
    h->ctx.artificial = scheme->artificial_type;
    h->ctx.ghost = scheme->ghost_species;
    for (int q = 0; q < 6; q++) h->ctx.bc[q] = block->Boundarys[q];
    h->ctx.glf = scheme->artificial_type == XFG_GLF ? (const double *)h->glf : nullptr;
    h->ctx.precision = scheme->precision;
    h->ctx.cfl = block->CFLnumber;
    h->ctx.viscous = scheme->viscous;
    for (int q = 0; q < 6; q++) g.bc[q] = block->Boundarys[q];
    if (h->fused && make_fused_tmaps(h)) {
        int nsm = 0;
        if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) == cudaSuccess && nsm > 0) {
            for (int q = 0; q < 3; q++) h->ctx.tmap[q] = &h->tmap[q];
            h->ctx.nsm = nsm;
        }
    }
    e = cudaMallocHost(&h->host_dtbuf, 8 * sizeof(double));
    if (e == cudaSuccess) e = cudaMallocHost(&h->host_err, 64 * sizeof(int));
    for (int q = 0; q < 4 && e == cudaSuccess; q++) e = cudaEventCreate(&h->ev[q]);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    if (e != cudaSuccess) {
        xfg_destroy(h);
        return fail(-2, "handle setup failed: %s", cudaGetErrorString(e));
    }
    *out = h;
    return 0;
}

int xfg_destroy(xfg_handle *h) {
    if (!h) return 0;
    cudaSetDevice(h->device);
    if (h->st) cudaStreamSynchronize(h->st);
    if (h->graph) cudaGraphExecDestroy(h->graph);
    for (int q = 0; q < 4; q++)
        if (h->ev[q]) cudaEventDestroy(h->ev[q]);
    if (h->pool) cudaFree(h->pool);
    if (h->host_dtbuf) cudaFreeHost(h->host_dtbuf);
    if (h->host_err) cudaFreeHost(h->host_err);
    if (h->st) cudaStreamDestroy(h->st);
    delete h;
    return 0;
}

static double *stage_U(xfg_handle *h, int flag) { return flag == 0 ? h->ctx.f.U : h->ctx.f.U1; }

int xfg_set_state(xfg_handle *h, const double *U_aos, const double *T) {
    if (!h || !U_aos) return fail(-1, "null argument");
    CK(cudaSetDevice(h->device));
    const size_t bytes = (size_t)h->N * h->E * sizeof(double);
    CK(cudaMemcpyAsync(h->stage, U_aos, bytes, cudaMemcpyDefault, h->st));
    const long long tot = h->N * h->E;
    k_aos_to_soa<<<grid_for(tot, 256), 256, 0, h->st>>>(h->stage, h->ctx.f.U, h->E, h->N, h->P);
    CK(cudaMemcpyAsync(h->ctx.f.U1, h->ctx.f.U, (size_t)h->P * h->E * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    // the fused stages' first output buffer starts as U1 does: ghost cells of a side whose fill does
    // nothing (Inflow; slip and viscous walls in y and z) keep the initial state, as U1's do
    if (h->fused)
        CK(cudaMemcpyAsync(h->ctx.f.U2, h->ctx.f.U, (size_t)h->P * h->E * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    if (T) CK(cudaMemcpyAsync(h->ctx.f.T, T, (size_t)h->N * sizeof(double), cudaMemcpyDefault, h->st));
    CK(cudaMemsetAsync(h->ctx.f.err, 0, 64 * sizeof(int), h->st));
    CK(cudaStreamSynchronize(h->st));
    h->states_ready = false;
    return 0;
}

// Device transport table of a viscous handle: the fitted ln(mu) and ln(kappa) cubics, the two
// species-pair factors of PHI (Visc_device.h:30-38) that depend on the molar masses only,
// (W_i/W_k)^0.25 and (1 + W_k/W_i)^-0.5, computed here once, and the species ids (SID).
int xfg_set_transport(xfg_handle *h, const xfg_transport *tr) {
    if (!h || !tr) return fail(-1, "null argument");
    if (!h->sc.viscous) return fail(-1, "the scheme has no viscous fluxes (xfg_scheme.viscous = 0)");
    std::vector<double> t;
    std::vector<float> tf;
    if (int rc = pack_transport(tr, h->NS, t, tf)) return rc;
    CK(cudaSetDevice(h->device));
    CK(cudaMemcpyAsync((void *)h->ctx.f.trf, tf.data(), tf.size() * sizeof(float), cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync((void *)h->ctx.f.tr, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
    h->transport_ready = true;
    return 0;
}

// Checkpoint file of XFLUIDS::Output_Ubak / Read_Ubak (src/XFLUIDS.cpp:658-724): int Step,
// double Time, float duration, then U in the reference layout (Emax doubles per cell, all cells
// with ghosts), packed, host byte order.
int xfg_checkpoint_write(xfg_handle *h, const char *path, int step, double time, float duration) {
    if (!h || !path) return fail(-1, "null argument");
    std::vector<double> U((size_t)h->N * h->E);
    int rc = xfg_get_array(h, XFG_U, U.data());
    if (rc) return rc;
    std::FILE *fp = std::fopen(path, "wb");
    if (!fp) return fail(-1, "cannot open %s for writing", path);
    bool ok = std::fwrite(&step, sizeof step, 1, fp) == 1 && std::fwrite(&time, sizeof time, 1, fp) == 1 &&
              std::fwrite(&duration, sizeof duration, 1, fp) == 1 &&
              std::fwrite(U.data(), sizeof(double), U.size(), fp) == U.size();
    ok = (std::fclose(fp) == 0) && ok;
    return ok ? 0 : fail(-1, "write of %s failed", path);
}

int xfg_checkpoint_read(xfg_handle *h, const char *path, int *step, double *time, float *duration) {
    if (!h || !path) return fail(-1, "null argument");
    std::FILE *fp = std::fopen(path, "rb");
    if (!fp) return fail(-1, "cannot open %s", path);
    int st = 0;
    double t = 0.0;
    float dur = 0.f;
    std::vector<double> U((size_t)h->N * h->E);
    bool ok = std::fread(&st, sizeof st, 1, fp) == 1 && std::fread(&t, sizeof t, 1, fp) == 1 &&
              std::fread(&dur, sizeof dur, 1, fp) == 1 && std::fread(U.data(), sizeof(double), U.size(), fp) == U.size();
    const bool extra = ok && std::fgetc(fp) != EOF;
    std::fclose(fp);
    if (!ok || extra)
        return fail(-1, "%s is not a checkpoint of this block (expected 16 + %zu bytes)", path, U.size() * sizeof(double));
    int rc = xfg_set_state(h, U.data(), nullptr);
    if (rc) return rc;
    h->t = t;
    if (step) *step = st;
    if (time) *time = t;
    if (duration) *duration = dur;
    return 0;
}

int xfg_get_array(xfg_handle *h, int which, double *out) {
    if (!h || !out) return fail(-1, "null argument");
    CK(cudaSetDevice(h->device));
    DevFields &f = h->ctx.f;
    const bool prim = which >= XFG_RHO && which <= XFG_E && which != XFG_T;
    if (prim && h->sc.precision == XFG_MIXED && !h->sc.cop)
        k_prims_from_primf<<<grid_for(h->N, 256), 256, 0, h->st>>>(h->ctx.g, f, h->sc.ncop_gamma);
    const double *src = nullptr;
    int comps = 1;
    switch (which) {
    case XFG_U: src = f.U, comps = h->E; break;
    case XFG_U1: src = f.U1, comps = h->E; break;
    case XFG_LU: src = f.LU, comps = h->E; break;
    case XFG_RHO: src = f.rho; break;
    case XFG_P: src = f.p; break;
    case XFG_U_VEL: src = f.u; break;
    case XFG_V_VEL: src = f.v; break;
    case XFG_W_VEL: src = f.w; break;
    case XFG_C: src = f.c; break;
    case XFG_H: src = f.H; break;
    case XFG_T: src = f.T; break;
    case XFG_GAMMA: src = f.gamma; break;
    case XFG_E: src = f.e; break;
    case XFG_CP: src = f.Cp; break;
    case XFG_R: src = f.R; break;
    case XFG_Y: src = f.y, comps = h->NS; break;
    case XFG_FWX: src = f.Fw[0], comps = h->E; break;
    case XFG_FWY: src = f.Fw[1], comps = h->E; break;
    case XFG_FWZ: src = f.Fw[2], comps = h->E; break;
    default: return fail(-1, "unknown array %d", which);
    }
    if (!src) return fail(-1, "array %d is not kept by this handle", which);
    if (comps == 1) {
        CK(cudaMemcpyAsync(out, src, (size_t)h->N * sizeof(double), cudaMemcpyDefault, h->st));
    } else {
        const long long tot = h->N * comps;
        k_soa_to_aos<<<grid_for(tot, 256), 256, 0, h->st>>>(src, h->stage, comps, h->N, h->P);
        CK(cudaMemcpyAsync(out, h->stage, (size_t)tot * sizeof(double), cudaMemcpyDefault, h->st));
    }
    CK(cudaStreamSynchronize(h->st));
    return 0;
}

int xfg_set_array(xfg_handle *h, int which, const double *in) {
    if (!h || !in) return fail(-1, "null argument");
    CK(cudaSetDevice(h->device));
    DevFields &f = h->ctx.f;
    if (which == XFG_T) {
        CK(cudaMemcpyAsync(f.T, in, (size_t)h->N * sizeof(double), cudaMemcpyDefault, h->st));
    } else if (which == XFG_U || which == XFG_U1) {
        const long long tot = h->N * h->E;
        CK(cudaMemcpyAsync(h->stage, in, (size_t)tot * sizeof(double), cudaMemcpyDefault, h->st));
        k_aos_to_soa<<<grid_for(tot, 256), 256, 0, h->st>>>(h->stage, which == XFG_U ? f.U : f.U1, h->E, h->N, h->P);
        CK(cudaGetLastError());
        if (which == XFG_U1 && h->fused)  // the stage-2 input buffer takes U1's ghost cells
            CK(cudaMemcpyAsync(f.U2, f.U1, (size_t)h->P * h->E * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    } else {
        return fail(-1, "array %d cannot be set (XFG_U, XFG_U1 or XFG_T)", which);
    }
    CK(cudaStreamSynchronize(h->st));
    return 0;
}

int xfg_boundary(xfg_handle *h, int flag) {
    if (!h) return fail(-1, "null handle");
    CK(cudaSetDevice(h->device));
    h->ops->bc(h->ctx, stage_U(h, flag), nullptr);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->st));
    return 0;
}

int xfg_update_states(xfg_handle *h, int flag, int *error, float *timers4) {
    if (!h) return fail(-1, "null handle");
    CK(cudaSetDevice(h->device));
    CK(cudaMemsetAsync(h->ctx.f.lam, 0, 3 * sizeof(unsigned long long), h->st));
    CK(cudaMemsetAsync(h->ctx.f.err + ERR_PRIM, 0, sizeof(int), h->st));
    CK(cudaEventRecord(h->ev[0], h->st));
    h->ops->states(h->ctx, stage_U(h, flag), 1, 0);
    CK(cudaGetLastError());
    CK(cudaEventRecord(h->ev[1], h->st));
    CK(cudaMemcpyAsync(h->host_err, h->ctx.f.err, 8 * sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    h->states_ready = true;
    if (error) *error = h->host_err[ERR_PRIM] ? 1 : 0;
    if (timers4) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]);
        timers4[0] = timers4[1] = timers4[2] = 0.f;
        timers4[3] = ms * 1e-3f;  // runtime_states, seconds like OutThisTime
    }
    return 0;
}

static void launch_lu(xfg_handle *h, double *UI, int guard) {
    const int dims[3] = {h->bl.DimX, h->bl.DimY, h->bl.DimZ};
    if (h->sc.artificial_type == XFG_GLF) h->ops->glf(h->ctx, h->glf, guard);
    for (int d = 0; d < 3; d++)
        if (dims[d]) h->ops->faces(h->ctx, d, UI, guard);
    if (h->sc.positivity)  // after all sweeps, ConVenction_block.hpp:328-410; lambda_0 in dtbuf[5..7]
        for (int d = 0; d < 3; d++)
            if (dims[d]) h->ops->pp(h->ctx, d, UI, h->ctx.f.dtbuf + 5, guard);
    if (h->sc.viscous) h->ops->visc(h->ctx, guard);  // ConVenction_block.hpp:419-566
}

int xfg_compute_lu(xfg_handle *h, int flag, float *timers23) {
    if (!h) return fail(-1, "null handle");
    if (h->sc.viscous && !h->transport_ready) return fail(-1, "viscous scheme: call xfg_set_transport first");
    CK(cudaSetDevice(h->device));
    CK(cudaEventRecord(h->ev[0], h->st));
    if (h->fused) {  // the fused stage recovers its own states and stores LU
        h->ops->fused(h->ctx, 0, stage_U(h, flag), nullptr, nullptr, nullptr, 0, 1, 0, 0);
        CK(cudaEventRecord(h->ev[1], h->st));
    } else {
        launch_lu(h, stage_U(h, flag), 0);
        CK(cudaEventRecord(h->ev[1], h->st));
        h->ops->div_rk(h->ctx, 0, 0.0, nullptr, 0, 1, 0);
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(h->ev[2], h->st));
    CK(cudaStreamSynchronize(h->st));
    if (timers23) {
        for (int q = 0; q < 23; q++) timers23[q] = 0.f;
        float a = 0.f, b = 0.f;
        cudaEventElapsedTime(&a, h->ev[0], h->ev[1]);
        cudaEventElapsedTime(&b, h->ev[1], h->ev[2]);
        timers23[11] = a * 1e-3f;  // runtime_flux
        timers23[22] = b * 1e-3f;  // runtime_updatelu
    }
    return 0;
}

int xfg_update_rk3(xfg_handle *h, int flag, double dt) {
    if (!h) return fail(-1, "null handle");
    if (flag < 1 || flag > 3) return fail(-1, "flag must be 1..3");
    CK(cudaSetDevice(h->device));
    h->ops->rk(h->ctx, flag, dt);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->st));
    return 0;
}

int xfg_get_dt(xfg_handle *h, double *dt) {
    if (!h || !dt) return fail(-1, "null argument");
    if (!h->states_ready) return fail(-1, "xfg_get_dt needs a preceding xfg_update_states");
    CK(cudaSetDevice(h->device));
    unsigned long long lam[3];
    CK(cudaMemcpyAsync(lam, h->ctx.f.lam, sizeof lam, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    double l[3];
    for (int q = 0; q < 3; q++) std::memcpy(&l[q], &lam[q], 8);
    const double dtref = l[0] * h->bl._dx + l[1] * h->bl._dy + l[2] * h->bl._dz;
    *dt = h->bl.CFLnumber / dtref;
    // the positivity limiter of the following stages uses these maxima (uvw_c_max, Fluids.cpp:899-908)
    CK(cudaMemcpyAsync(h->ctx.f.dtbuf + 5, l, sizeof l, cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
    return 0;
}

int xfg_estimate_nan(xfg_handle *h, int flag, int *error, int *error_pos) {
    if (!h) return fail(-1, "null handle");
    CK(cudaSetDevice(h->device));
    int *pos = h->ctx.f.err + 16;  // scratch after the error words
    CK(cudaMemsetAsync(pos, 0, 40 * sizeof(int), h->st));
    const double *UI = (flag == 1 || flag == 2) ? h->ctx.f.U1 : h->ctx.f.U;  // src/Fluids.cpp:966-983
    h->ops->estimate_nan(h->ctx, UI, pos);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h->host_err + 16, pos, 40 * sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    const int *hp = h->host_err + 16;
    const int E = h->E;
    if (error) *error = hp[E] ? 1 : 0;
    if (error_pos) {
        for (int n = 0; n < E; n++) error_pos[n] = hp[n];
        error_pos[E] = 0;
        for (int q = 1; q <= 3; q++) error_pos[E + q] = hp[E + q];
    }
    return hp[E] ? 10000 : 0;
}

// The launches of one fused step, all guarded by the device "done" flag so that replays past
// the target time do nothing.
static void launch_step(xfg_handle *h) {
    DevFields &f = h->ctx.f;
    k_dt_step<<<1, 1, 0, h->st>>>(h->ctx.g, f, h->bl.CFLnumber);
    if (h->fused) {
        // U -> U2 -> U1 -> U: a stage never writes the array its tiles read as halo; U1 ends as
        // the second stage's result, as in the reference
        h->ops->bc(h->ctx, f.U, f.dtbuf);
        h->ops->fused(h->ctx, 1, f.U, nullptr, f.U2, f.dtbuf, 1, 0, 0, 1);
        h->ops->bc(h->ctx, f.U2, f.dtbuf);
        h->ops->fused(h->ctx, 2, f.U2, f.U, f.U1, f.dtbuf, 1, 0, 0, 1);
        h->ops->bc(h->ctx, f.U1, f.dtbuf);
        h->ops->fused_ghost_lam(h->ctx, f.U1, 1);
        h->ops->fused(h->ctx, 3, f.U1, f.U, f.U, f.dtbuf, 1, 0, 1, 1);
        return;
    }
    for (int flag = 1; flag <= 3; flag++) {
        double *UI = flag == 1 ? f.U : f.U1;
        h->ops->bc(h->ctx, UI, f.dtbuf);
        h->ops->states(h->ctx, UI, flag == 3 ? 1 : 0, 1);
        launch_lu(h, UI, 1);
        h->ops->div_rk(h->ctx, flag, 0.0, f.dtbuf, 1, 0, 1);
    }
}

static int finish(xfg_handle *h, double *t, double *dt, int *steps) {
    CK(cudaMemcpyAsync(h->host_dtbuf, h->ctx.f.dtbuf, 8 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaMemcpyAsync(h->host_err, h->ctx.f.err, 8 * sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    h->t = h->host_dtbuf[1];
    if (t) *t = h->t;
    if (dt) *dt = h->host_dtbuf[0];
    if (steps) *steps = (int)h->host_dtbuf[3];
    if (h->host_err[ERR_TMA]) return fail(-2, "a TMA copy of the fused stage did not complete");
    if (h->host_err[ERR_STATE]) return 10000;
    if (h->host_err[ERR_PRIM]) return 1;
    return 0;
}

int xfg_step(xfg_handle *h, double target_t, double *t, double *dt) {
    if (!h) return fail(-1, "null handle");
    if (!h->states_ready) return fail(-1, "xfg_step needs a preceding xfg_update_states (main.cpp:45-47)");
    if (h->sc.viscous && !h->transport_ready) return fail(-1, "viscous scheme: call xfg_set_transport first");
    CK(cudaSetDevice(h->device));
    k_set_time<<<1, 1, 0, h->st>>>(h->ctx.f.dtbuf, h->t, target_t);
    launch_step(h);
    CK(cudaGetLastError());
    return finish(h, t, dt, nullptr);
}

static int advance_impl(xfg_handle *h, int nsteps, double target_t, double *t, int *steps_done, float *device_ms);

int xfg_advance(xfg_handle *h, int nsteps, double target_t, double *t, int *steps_done) {
    return advance_impl(h, nsteps, target_t, t, steps_done, nullptr);
}

int xfg_advance_timed(xfg_handle *h, int nsteps, double target_t, double *t, int *steps_done, float *device_ms) {
    return advance_impl(h, nsteps, target_t, t, steps_done, device_ms);
}

static int advance_impl(xfg_handle *h, int nsteps, double target_t, double *t, int *steps_done, float *device_ms) {
    if (!h) return fail(-1, "null handle");
    if (!h->states_ready) return fail(-1, "xfg_advance needs a preceding xfg_update_states (main.cpp:45-47)");
    if (h->sc.viscous && !h->transport_ready) return fail(-1, "viscous scheme: call xfg_set_transport first");
    CK(cudaSetDevice(h->device));
    k_set_time<<<1, 1, 0, h->st>>>(h->ctx.f.dtbuf, h->t, target_t);
    CK(cudaGetLastError());
    if (!h->graph) {
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
        launch_step(h);
        cudaError_t e = cudaStreamEndCapture(h->st, &g);
        if (e != cudaSuccess) return fail(-2, "graph capture failed: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&h->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(-2, "graph instantiate failed: %s", cudaGetErrorString(e));
    }
    if (device_ms) CK(cudaEventRecord(h->ev[2], h->st));
    for (int s = 0; s < nsteps; s++) CK(cudaGraphLaunch(h->graph, h->st));
    if (device_ms) CK(cudaEventRecord(h->ev[3], h->st));
    int rc = finish(h, t, nullptr, steps_done);
    if (device_ms) cudaEventElapsedTime(device_ms, h->ev[2], h->ev[3]);
    return rc;
}

int xfg_pinned_alloc(size_t bytes, void **ptr) {
    if (!ptr) return fail(-1, "null argument");
    CK(cudaMallocHost(ptr, bytes));
    return 0;
}

int xfg_pinned_free(void *ptr) {
    CK(cudaFreeHost(ptr));
    return 0;
}

int xfg_launches_per_step(xfg_handle *h, int *n) {
    if (!h || !n) return fail(-1, "null argument");
    const int dims = h->bl.DimX + h->bl.DimY + h->bl.DimZ;
    const int glf = h->sc.artificial_type == XFG_GLF ? 1 : 0;
    *n = 1 + 3 * (dims + 1 + glf + dims + 1);  // dt, then per stage: bc per dim, states, [glf], faces per dim, div+rk
    if (h->fused) *n = 1 + 3 * (dims + 1) + 1;  // dt, per stage: bc per dim, the fused stage; ghost maxima
    return 0;
}

// Per-phase device times of one fused step (ms, summed over the 3 stages): [0] dt, [1] boundary,
// [2] states, [3..5] faces x/y/z, [6] divergence + RK. Events on the handle's stream.
int xfg_time_phases(xfg_handle *h, double target_t, float *ms_out) {
    if (!h || !ms_out) return fail(-1, "null argument");
    if (!h->states_ready) return fail(-1, "xfg_time_phases needs a preceding xfg_update_states");
    if (h->sc.viscous && !h->transport_ready) return fail(-1, "viscous scheme: call xfg_set_transport first");
    CK(cudaSetDevice(h->device));
    DevFields &f = h->ctx.f;
    const int dims[3] = {h->bl.DimX, h->bl.DimY, h->bl.DimZ};
    cudaEvent_t ev[32];
    int ne = 0;
    for (int q = 0; q < 32; q++) CK(cudaEventCreate(&ev[q]));
    int phase_of[32];
    k_set_time<<<1, 1, 0, h->st>>>(f.dtbuf, h->t, target_t);
    CK(cudaEventRecord(ev[ne++], h->st));
    k_dt_step<<<1, 1, 0, h->st>>>(h->ctx.g, f, h->bl.CFLnumber);
    phase_of[ne] = 0;
    CK(cudaEventRecord(ev[ne++], h->st));
    // fused stages: [1] boundary (+ ghost-cell dt maxima), [3] the fused stage kernel
    double *const fin[3] = {f.U, f.U2, f.U1}, *const fout[3] = {f.U2, f.U1, f.U};
    for (int flag = 1; flag <= 3 && h->fused; flag++) {
        h->ops->bc(h->ctx, fin[flag - 1], f.dtbuf);
        if (flag == 3) h->ops->fused_ghost_lam(h->ctx, f.U1, 1);
        phase_of[ne] = 1;
        CK(cudaEventRecord(ev[ne++], h->st));
        h->ops->fused(h->ctx, flag, fin[flag - 1], f.U, fout[flag - 1], f.dtbuf, 1, 0, flag == 3, 1);
        phase_of[ne] = 3;
        CK(cudaEventRecord(ev[ne++], h->st));
    }
    for (int flag = 1; flag <= 3 && !h->fused; flag++) {
        double *UI = flag == 1 ? f.U : f.U1;
        h->ops->bc(h->ctx, UI, f.dtbuf);
        phase_of[ne] = 1;
        CK(cudaEventRecord(ev[ne++], h->st));
        h->ops->states(h->ctx, UI, flag == 3 ? 1 : 0, 1);
        phase_of[ne] = 2;
        CK(cudaEventRecord(ev[ne++], h->st));
        if (h->sc.artificial_type == XFG_GLF) h->ops->glf(h->ctx, h->glf, 1);
        for (int d = 0; d < 3; d++)
            if (dims[d]) {
                h->ops->faces(h->ctx, d, UI, 1);
                phase_of[ne] = 3 + d;
        CK(cudaEventRecord(ev[ne++], h->st));
            }
        h->ops->div_rk(h->ctx, flag, 0.0, f.dtbuf, 1, 0, 1);
        phase_of[ne] = 6;
        CK(cudaEventRecord(ev[ne++], h->st));
    }
    CK(cudaGetLastError());
    int rc = finish(h, nullptr, nullptr, nullptr);
    for (int q = 0; q < 7; q++) ms_out[q] = 0.f;
    for (int q = 1; q < ne; q++) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[q - 1], ev[q]);
        ms_out[phase_of[q]] += ms;
    }
    for (int q = 0; q < 32; q++) cudaEventDestroy(ev[q]);
    return rc < 0 ? rc : 0;
}

int xfg_set_time(xfg_handle *h, double t) {
    if (!h) return fail(-1, "null handle");
    h->t = t;
    return 0;
}
int xfg_get_time(xfg_handle *h, double *t) {
    if (!h || !t) return fail(-1, "null argument");
    *t = h->t;
    return 0;
}
int xfg_synchronize(xfg_handle *h) {
    if (!h) return fail(-1, "null handle");
    CK(cudaSetDevice(h->device));
    CK(cudaStreamSynchronize(h->st));
    return 0;
}
int xfg_device_array(xfg_handle *h, int which, double **ptr, size_t *pitch) {
    if (!h || !ptr) return fail(-1, "null argument");
    DevFields &f = h->ctx.f;
    double *a = nullptr;
    switch (which) {
    case XFG_U: a = f.U; break;
    case XFG_U1: a = f.U1; break;
    case XFG_LU: a = f.LU; break;
    case XFG_RHO: a = f.rho; break;
    case XFG_P: a = f.p; break;
    case XFG_T: a = f.T; break;
    default: return fail(-1, "array %d has no device view", which);
    }
    *ptr = a;
    if (pitch) *pitch = (size_t)h->P;
    return 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// FMA throughput probe (roofline denominators of the compute-bound kernels)
// ---------------------------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256) k_fma_chain(T *out, int iters, T a, T b) {
    T x0 = (T)threadIdx.x, x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
    T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 8; u++) {
            x0 = fma(x0, a, b), x1 = fma(x1, a, b), x2 = fma(x2, a, b), x3 = fma(x3, a, b);
            x4 = fma(x4, a, b), x5 = fma(x5, a, b), x6 = fma(x6, a, b), x7 = fma(x7, a, b);
        }
    }
    T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == T(-1.2345)) out[threadIdx.x] = s;  // keeps the chain live
}

template <class T>
static double run_fma(int sms, int iters, cudaStream_t st, T *scratch) {
    const int blocks = sms * 8, threads = 256;
    cudaEvent_t a, b;
    cudaEventCreate(&a), cudaEventCreate(&b);
    k_fma_chain<T><<<blocks, threads, 0, st>>>(scratch, iters / 8, T(0.999999), T(1e-7));  // warm-up
    cudaEventRecord(a, st);
    k_fma_chain<T><<<blocks, threads, 0, st>>>(scratch, iters, T(0.999999), T(1e-7));
    cudaEventRecord(b, st);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a), cudaEventDestroy(b);
    const double flops = 2.0 * 8.0 * 8.0 * (double)iters * blocks * threads;
    return flops / (ms * 1e-3);
}

extern "C" int xfg_measure_pipe_peaks(int device, double *out) {
    if (!out) return fail(-1, "null out");
    CK(cudaSetDevice(device));
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    void *scratch;
    CK(cudaMalloc(&scratch, 256 * sizeof(double)));
    out[0] = run_fma<double>(sms, 2048, st, (double *)scratch);
    out[1] = run_fma<float>(sms, 65536, st, (float *)scratch);
    int clk = 0;
    cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, device);
    out[2] = clk / 1000.0;
    cudaError_t e = cudaGetLastError();
    cudaFree(scratch);
    cudaStreamDestroy(st);
    if (e != cudaSuccess) return fail(-2, "peak probe failed: %s", cudaGetErrorString(e));
    return 0;
}
