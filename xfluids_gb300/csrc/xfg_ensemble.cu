// xfg_ensemble.cu - many independent single-gas grids advanced together (batched ensemble and the
// device side of the request server).
//
// All members live in one device pool (allocated once; members are sub-allocated first-fit, so
// admission is by HBM budget). One step of every active member is one sequence of batched kernels:
// each launch covers the blocks of all members of that phase, a block finds its member through a
// prefix table of block offsets and runs the same device bodies as the single-grid kernels
// (xfg_kernels.cuh / xfg_mixed.cuh) on that member's arrays. Every member has its own dt, time,
// target time and done flag on the device; members that reached their target skip all work. The
// step is captured once in a CUDA graph and replayed until membership changes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/xfluids_gb300.h"
#define XFG_KNS ens
#include "xfg_ensemble.cuh"

using namespace xfg;
using namespace xfg::ens;

namespace xfg {
// ensemble launcher registry (xfg_ensemble.cuh)
static std::vector<EnsOps> &ens_registry() {
    static std::vector<EnsOps> r;
    return r;
}
void register_ens_ops(const EnsOps *ops) {
    for (EnsOps &o : ens_registry())
        if (o.cop == ops->cop && o.ns == ops->ns && o.precision == ops->precision) {
            auto faces = o.faces;
            auto faces_all = o.faces_all;
            const bool overridden = o.bc == nullptr;  // a face override registered first
            o = *ops;
            if (overridden) o.faces = faces, o.faces_all = faces_all;
            return;
        }
    ens_registry().push_back(*ops);
}
void register_ens_faces(int cop, int ns, int precision, decltype(EnsOps::faces) faces,
                        decltype(EnsOps::faces_all) faces_all) {
    for (EnsOps &o : ens_registry())
        if (o.cop == cop && o.ns == ns && o.precision == precision) {
            o.faces = faces, o.faces_all = faces_all;
            return;
        }
    EnsOps o{};
    o.cop = cop, o.ns = ns, o.precision = precision, o.faces = faces, o.faces_all = faces_all;
    ens_registry().push_back(o);
}
const EnsOps *find_ens_ops(int cop, int ns, int precision) {
    for (const EnsOps &o : ens_registry())
        if (o.cop == cop && o.ns == ns && o.precision == precision && o.bc) return &o;
    return nullptr;
}
}  // namespace xfg

// the single-gas tables (mixtures: xfg_ensemble_cop<N>*.cu)
static EnsRegistrar<false, 1, false> reg_fp64(XFG_FP64);
static EnsRegistrar<false, 1, true> reg_mixed(XFG_MIXED);

namespace {

using Member = EnsMember;

// size classes with their own face tile: 1D, 2D below 384 cells per side, 2D from 384, 3D
enum { CL_1D, CL_2D_SMALL, CL_2D_LARGE, CL_3D, CL_N };

// One stage of the fused members: CTA = one 32 x 7 tile of one member (fused_stage_tile), stage
// buffers U -> U2 -> U1 -> U as in the single-grid fused step.
template <bool LLF>
__global__ void __launch_bounds__(fz::THREADS, 2)
    kb_fused(const Member *__restrict__ M, const int *__restrict__ off, int n, FusedK k, int flag) {
    const int mi = member_of_block(off, n, blockIdx.x);
    if (member_done(M[mi])) return;
    // local copies of the member's geometry and arrays: the tile's stores cannot alias them, so
    // they stay in registers, and the arrays are global memory (global, not generic, accesses)
    const Geo g = M[mi].g;
    const DevFields f = M[mi].f;
    __builtin_assume(__isGlobal(f.U) && __isGlobal(f.U1) && __isGlobal(f.U2) && __isGlobal(f.primf));
    __builtin_assume(__isGlobal(f.lam) && __isGlobal(f.err) && __isGlobal(f.dtbuf));
    const int lb = blockIdx.x - off[mi], tx = (g.Xi + fz::TX - 1) / fz::TX;
    const double *UI = flag == 1 ? f.U : (flag == 2 ? f.U2 : f.U1);
    double *Uout = flag == 1 ? f.U2 : (flag == 2 ? f.U1 : f.U);
    fused_stage_tile<LLF>(g, f, k, UI, f.U, Uout, flag, f.dtbuf[0], 1, 0, flag == 3, lb % tx, lb / tx);
}
__global__ void __launch_bounds__(kThreads) kb_fused_ghost(const Member *__restrict__ M, const int *__restrict__ off,
                                                           int n, float gamma) {
    const int mi = member_of_block(off, n, blockIdx.x);
    const Member &m = M[mi];
    if (member_done(m)) return;
    fused_ghost_lam_body(m.g, m.f, gamma, m.f.U1, (long long)(blockIdx.x - off[mi]) * blockDim.x + threadIdx.x);
}

__global__ void kb_dt(const Member *__restrict__ M, int n) {
    const int mi = blockIdx.x * blockDim.x + threadIdx.x;
    if (mi >= n) return;
    const Member &m = M[mi];
    if (!m.active) return;
    // a member whose last step produced a NaN / Inf / negative density or pressure stops there,
    // as the reference's run stops after EstimateFluidNAN / UpdateFluidStates report an error
    if (m.f.err[ERR_STATE] | m.f.err[ERR_PRIM]) {
        if (m.f.dtbuf[4] == 0.0) m.f.dtbuf[4] = 2.0, m.f.dtbuf[0] = 0.0;
        return;
    }
    dt_step_body(m.g, m.f, m.cfl);
}

__global__ void kb_aos_to_soa(const double *__restrict__ aos, double *__restrict__ soa, int E, long long N, long long P) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * E) return;
    soa[(t % E) * P + t / E] = aos[t];
}
__global__ void kb_soa_to_aos(const double *__restrict__ soa, double *__restrict__ aos, int E, long long N, long long P) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * E) return;
    aos[t] = soa[(t % E) * P + t / E];
}

size_t up(size_t x, size_t a) { return (x + a - 1) / a * a; }

thread_local std::string g_eerr;
int efail(int code, const char *fmt, const char *detail = "") {  // fmt takes one %s
    char buf[512];
    snprintf(buf, sizeof buf, fmt, detail);
    set_last_error(buf);
    return code;
}
#define ECK(call)                                                                            \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) return efail(-2, #call " failed: %s", cudaGetErrorString(e_)); \
    } while (0)

// First-fit allocator over the device pool (offsets in bytes).
struct PoolAlloc {
    size_t size = 0;
    std::map<size_t, size_t> free_;  // offset -> length
    void init(size_t n) { size = n, free_.clear(), free_[0] = n; }
    bool alloc(size_t n, size_t *off) {
        n = up(n, 256);
        for (auto it = free_.begin(); it != free_.end(); ++it)
            if (it->second >= n) {
                *off = it->first;
                size_t rest = it->second - n, o = it->first + n;
                free_.erase(it);
                if (rest) free_[o] = rest;
                return true;
            }
        return false;
    }
    void release(size_t off, size_t n) {
        n = up(n, 256);
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) it->second += nx->second, free_.erase(nx);
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) pv->second += it->second, free_.erase(it);
        }
    }
    size_t free_bytes() const {
        size_t s = 0;
        for (auto &kv : free_) s += kv.second;
        return s;
    }
};

}  // namespace

struct xfg_ensemble {
    int device = 0;
    cudaStream_t st = nullptr;
    xfg_scheme sc;
    DevThermo th;
    int capacity = 0;
    char *pool = nullptr;
    size_t pool_bytes = 0;
    PoolAlloc alloc;
    std::vector<Member> hm;               // host mirror of the member table
    std::vector<size_t> m_off, m_len;     // pool allocation of each slot
    std::vector<xfg_block> blocks;
    Member *dm = nullptr;                 // device member table
    int *doff = nullptr;                  // device block tables, PH_N rows of 3 capacity + 1
    double *ddt = nullptr;                // device dtbuf of all slots (8 doubles each)
    double *hdt = nullptr;                // pinned mirror
    int *derr = nullptr;                  // device error words (8 ints each)
    double *dhsc = nullptr;               // mixtures: the scaled enthalpy tables (DevThermo::hsc)
    double *dtr = nullptr;                // viscous mixtures: transport tables, FP64 then FP32
    float *dtrf = nullptr;
    bool transport_ready = false;         // xfg_ensemble_set_transport called
    int *herr = nullptr;
    std::vector<int> order;               // active slots in launch order
    int nblk[PH_N] = {0};
    bool dirty = true;
    cudaGraphExec_t graph = nullptr;
    int graph_built_steps = 0;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    // launch schedule (xfg_ensemble_set_option)
    int largest_first = 1;
    int fused_faces = 0;                  // one launch for all face sweeps
    int graph_steps = 1;                  // fused steps per captured graph
    int ltx[CL_N] = {7, 5, 5, 5};         // face tile per size class
    bool fused_ok = false;                // mixed WENO5 LLF / Roe without limiter: 2D members fused
    FusedK fk{};
    const EnsOps *ops = nullptr;          // batched launchers of the ensemble's gas model and form
    int E = 5, NS = 1;
};

namespace {

size_t row_len(const xfg_ensemble *e) { return 3 * (size_t)e->capacity + 1; }

bool two_d(const xfg_block &b) { return b.DimX && b.DimY && !b.DimZ; }

// Device bytes of one member: the single-grid arrays of its gas model (ns species, 1 for a single
// gas) and form, as xfg_create lays them out (viscous mixtures: the velocity derivatives, mu and
// kappa), without the transpose arrays.
size_t member_bytes(const xfg_block &b, int cop, int ns, bool mixed, int visc) {
    const size_t N = (size_t)b.Xmax * b.Ymax * b.Zmax, P = up(N, 64);
    const int dims = b.DimX + b.DimY + b.DimZ, E = cop ? ns + 4 : 5;
    size_t nd = 3 * E + 12;                                    // U, U1, LU, primitives
    if (cop) nd += ns + (mixed ? 0 : 3 + (ns - 1));           // y, per-cell sound-speed terms (FP64 form)
    if (mixed && !cop && two_d(b)) nd += 5;                    // U2 of the fused stages
    if (!mixed) nd += 2 * E * dims + (cop ? 0 : 2 + 3 * dims); // F, Fw; single gas: sqrt(rho), 1/sqrt(rho), |lambda|
    size_t bytes = nd * P * 8;
    if (mixed) bytes += (size_t)(E + 7 + 2 * E * dims + (cop ? ns + 3 + (ns - 1) : 0) + (visc ? 9 + 3 : 0)) * up(P * 4, 256);
    if (visc && !mixed) bytes += (size_t)(9 + 2) * P * 8;
    return bytes + 1024;                                       // lam + small words
}

void carve(Member &m, char *base, const xfg_block &b, int cop, int ns, bool mixed, int visc, const double *tr,
           const float *trf) {
    const size_t N = (size_t)b.Xmax * b.Ymax * b.Zmax, P = up(N, 64);
    const int dims[3] = {b.DimX, b.DimY, b.DimZ}, E = cop ? ns + 4 : 5;
    char *p = base;
    auto t8 = [&](int c) { double *r = (double *)p; p += (size_t)c * P * 8; return r; };
    auto t4 = [&](int c) { float *r = (float *)p; p += (size_t)c * up(P * 4, 256); return r; };
    DevFields &f = m.f;
    std::memset(&f, 0, sizeof f);
    f.U = t8(E), f.U1 = t8(E), f.LU = t8(E);
    if (mixed && !cop && two_d(b)) f.U2 = t8(5);
    f.rho = t8(1), f.u = t8(1), f.v = t8(1), f.w = t8(1), f.p = t8(1), f.H = t8(1);
    f.c = t8(1), f.T = t8(1), f.gamma = t8(1), f.e = t8(1), f.Cp = t8(1), f.R = t8(1);
    if (cop) f.y = t8(ns);
    if (cop && !mixed) f.xc = t8(3 + (ns - 1));
    if (!mixed) {
        for (int d = 0; d < 3; d++)
            if (dims[d]) f.F[d] = t8(E), f.Fw[d] = t8(E);
        if (!cop) {
            f.sr = t8(1), f.isr = t8(1);
            for (int d = 0; d < 3; d++)
                if (dims[d]) f.eab[d] = t8(3);
        }
        if (visc) f.vde = t8(9), f.mu = t8(1), f.kappa = t8(1);
    } else {
        f.Uf = t4(E), f.primf = t4(7);
        if (cop) f.yf = t4(ns), f.xcf = t4(3 + (ns - 1));
        if (visc) f.vdef = t4(9), f.muf = t4(1), f.kappaf = t4(1), f.Tf = t4(1);
        for (int d = 0; d < 3; d++)
            if (dims[d]) f.Ff[d] = t4(E), f.Fwf[d] = t4(E);
    }
    if (visc) f.tr = tr, f.trf = trf;  // the ensemble's transport tables
    m.visc = visc;
    f.lam = (unsigned long long *)p;
    m.glf = (unsigned long long *)(p + 64);
    Geo &g = m.g;
    g.Xmax = b.Xmax, g.Ymax = b.Ymax, g.Zmax = b.Zmax, g.Xi = b.X_inner, g.Yi = b.Y_inner, g.Zi = b.Z_inner;
    g.Bx = b.Bwidth_X, g.By = b.Bwidth_Y, g.Bz = b.Bwidth_Z, g.dimx = b.DimX, g.dimy = b.DimY, g.dimz = b.DimZ;
    g._dx = b._dx, g._dy = b._dy, g._dz = b._dz, g.pitch = (long long)P;
    geo_split_spacing(g);
    g.dx = b.dx, g.dy = b.dy, g.dz = b.dz;
    for (int q = 0; q < 6; q++) g.bc[q] = b.Boundarys[q];
    m.cfl = b.CFLnumber;
    for (int q = 0; q < 6; q++) m.bc[q] = b.Boundarys[q];
}

int size_class(const Geo &g) {
    const int dims = g.dimx + g.dimy + g.dimz;
    if (dims == 1) return CL_1D;
    if (dims == 3) return CL_3D;
    return std::max(g.Xi, std::max(g.Yi, g.Zi)) < 384 ? CL_2D_SMALL : CL_2D_LARGE;
}

int face_blocks(const Geo &g, int d, int ltx) {
    const int dims[3] = {g.dimx, g.dimy, g.dimz};
    if (!dims[d]) return 0;
    const dim3 b = d == 0 ? face_grid_tile<0>(g, ltx) : (d == 1 ? face_grid_tile<1>(g, ltx) : face_grid_tile<2>(g, ltx));
    return (int)(b.x * b.y * b.z);
}

int blocks_of(const Member &m, int ph, int ltx) {
    const Geo &g = m.g;
    const long long N = g.ncell(), inner = (long long)g.Xi * g.Yi * g.Zi;
    auto gb = [](long long n) { return (int)((n + kThreads - 1) / kThreads); };
    if (ph == PH_FUSED)
        return m.fused ? ((g.Xi + fz::TX - 1) / fz::TX) * ((g.Yi + fz::TY - 1) / fz::TY) : 0;
    if (ph == PH_GLAM) return m.fused ? gb(fused_ghost_cells(g)) : 0;
    if (ph >= PH_VCELL && ph <= PH_VF2) {
        if (!m.visc) return 0;
        const int dims[3] = {g.dimx, g.dimy, g.dimz};
        if (ph == PH_VCELL)
            return gb((long long)(g.dimx ? g.Xi + 4 : 1) * (g.dimy ? g.Yi + 4 : 1) * (g.dimz ? g.Zi + 4 : 1));
        if (ph <= PH_VBC2) {
            const int d = ph - PH_VBC0;
            const long long nb[3] = {(long long)g.Bx * g.Ymax * g.Zmax, (long long)g.By * g.Xmax * g.Zmax,
                                     (long long)g.Bz * g.Xmax * g.Ymax};
            return dims[d] ? gb(nb[d]) : 0;
        }
        const int d = ph - PH_VF0;
        const long long nf[3] = {(long long)(g.Xi + 1) * g.Yi * g.Zi, (long long)g.Xi * (g.Yi + 1) * g.Zi,
                                 (long long)g.Xi * g.Yi * (g.Zi + 1)};
        return dims[d] ? gb(nf[d]) : 0;
    }
    if (m.fused && ph >= PH_STATES && ph <= PH_DIV) return 0;  // done by the fused tiles
    switch (ph) {
    case PH_BC0: return g.dimx ? gb((long long)g.Bx * g.Ymax * g.Zmax) : 0;
    case PH_BC1: return g.dimy ? gb((long long)g.By * g.Xmax * g.Zmax) : 0;
    case PH_BC2: return g.dimz ? gb((long long)g.Bz * g.Xmax * g.Ymax) : 0;
    case PH_STATES: return gb(N);
    case PH_F0: return face_blocks(g, 0, ltx);
    case PH_F1: return face_blocks(g, 1, ltx);
    case PH_F2: return face_blocks(g, 2, ltx);
    case PH_DIV: return gb(inner);
    }
    return 0;
}

// Rebuild the launch order, the block tables and the device member table.
int rebuild(xfg_ensemble *e) {
    e->order.clear();
    for (int s = 0; s < e->capacity; s++)
        if (e->hm[s].active) e->order.push_back(s);
    if (e->largest_first)
        std::stable_sort(e->order.begin(), e->order.end(), [e](int a, int b) { return e->hm[a].g.ncell() > e->hm[b].g.ncell(); });
    const int n = (int)e->order.size();
    std::vector<Member> ordered(std::max(n, 1));
    for (int q = 0; q < n; q++) {
        ordered[q] = e->hm[e->order[q]];
        ordered[q].ltx = e->ltx[size_class(ordered[q].g)];
    }
    std::vector<int> tab((size_t)PH_N * row_len(e), 0);
    for (int ph = 0; ph < PH_N; ph++) {
        long long acc = 0;
        int *t = &tab[(size_t)ph * row_len(e)];
        if (ph == PH_FALL) {
            for (int q = 0; q < n; q++)
                for (int d = 0; d < 3; d++)
                    t[3 * q + d] = (int)acc, acc += ordered[q].fused ? 0 : face_blocks(ordered[q].g, d, ordered[q].ltx);
            t[3 * n] = (int)acc;
        } else {
            for (int q = 0; q < n; q++) t[q] = (int)acc, acc += blocks_of(ordered[q], ph, ordered[q].ltx);
            t[n] = (int)acc;
        }
        if (acc > 0x7fffffffLL) return efail(-1, "ensemble too large for one launch per phase%s");
        e->nblk[ph] = (int)acc;
    }
    ECK(cudaMemcpyAsync(e->dm, ordered.data(), sizeof(Member) * std::max(n, 1), cudaMemcpyHostToDevice, e->st));
    ECK(cudaMemcpyAsync(e->doff, tab.data(), sizeof(int) * tab.size(), cudaMemcpyHostToDevice, e->st));
    ECK(cudaStreamSynchronize(e->st));
    if (e->graph) cudaGraphExecDestroy(e->graph), e->graph = nullptr;
    e->dirty = false;
    return 0;
}

const int *tab(const xfg_ensemble *e, int ph) { return e->doff + (size_t)ph * row_len(e); }

void launch_step(xfg_ensemble *e) {
    const int n = (int)e->order.size();
    if (!n) return;
    const EnsOps *ops = e->ops;
    const int order = e->sc.scheme_order, art = e->sc.artificial_type;
    cudaStream_t st = e->st;
    kb_dt<<<(n + 127) / 128, 128, 0, st>>>(e->dm, n);
    for (int flag = 1; flag <= 3; flag++) {
        for (int d = 0; d < 3; d++)
            if (e->nblk[PH_BC0 + d]) ops->bc(e->dm, tab(e, PH_BC0 + d), e->nblk[PH_BC0 + d], n, d, flag, st);
        if (e->nblk[PH_FUSED]) {  // fused members: one launch for the whole stage
            if (flag == 3 && e->nblk[PH_GLAM])
                kb_fused_ghost<<<e->nblk[PH_GLAM], kThreads, 0, st>>>(e->dm, tab(e, PH_GLAM), n, e->fk.gamma);
            if (art == XFG_LLF)
                kb_fused<true><<<e->nblk[PH_FUSED], fz::THREADS, sizeof(FusedTile), st>>>(e->dm, tab(e, PH_FUSED), n, e->fk, flag);
            else
                kb_fused<false><<<e->nblk[PH_FUSED], fz::THREADS, sizeof(FusedTile), st>>>(e->dm, tab(e, PH_FUSED), n, e->fk, flag);
        }
        if (!e->nblk[PH_STATES]) continue;  // no member left on the separate stage kernels
        ops->states(e->dm, tab(e, PH_STATES), e->nblk[PH_STATES], n, e->th, e->sc.ghost_species, flag, flag == 3, st);
        if (art == XFG_GLF) ops->glf(e->dm, tab(e, PH_STATES), e->nblk[PH_STATES], n, st);
        if (e->fused_faces) {
            if (e->nblk[PH_FALL]) ops->faces_all(e->dm, tab(e, PH_FALL), e->nblk[PH_FALL], 3 * n, e->th, order, flag, art, st);
        } else {
            for (int d = 0; d < 3; d++)
                if (e->nblk[PH_F0 + d])
                    ops->faces(e->dm, tab(e, PH_F0 + d), e->nblk[PH_F0 + d], n, e->th, d, order, flag, art, st);
        }
        if (e->sc.positivity) ops->pp(e->dm, tab(e, PH_DIV), e->nblk[PH_DIV], n, flag, st);
        if (e->sc.viscous && e->nblk[PH_VCELL]) {  // ConVenction_block.hpp:419-566, the single grid's order
            const int heat = (e->sc.viscous & 2) ? 1 : 0;
            ops->vderiv(e->dm, tab(e, PH_VCELL), e->nblk[PH_VCELL], n, st);
            for (int d = 0; d < 3; d++)
                if (e->nblk[PH_VBC0 + d]) ops->vderiv_bc(e->dm, tab(e, PH_VBC0 + d), e->nblk[PH_VBC0 + d], n, d, st);
            ops->transport(e->dm, tab(e, PH_VCELL), e->nblk[PH_VCELL], n, e->th, heat, st);
            for (int d = 0; d < 3; d++)
                if (e->nblk[PH_VF0 + d]) ops->visc(e->dm, tab(e, PH_VF0 + d), e->nblk[PH_VF0 + d], n, d, heat, st);
        }
        ops->div_rk(e->dm, tab(e, PH_DIV), e->nblk[PH_DIV], n, flag, st);
    }
}

}  // namespace

extern "C" {

int xfg_ensemble_create(int capacity, size_t pool_bytes, const xfg_scheme *scheme, const xfg_thermal *thermal,
                        int device, xfg_ensemble **out) {
    if (!out || !scheme || capacity <= 0) return efail(-1, "bad argument%s");
    *out = nullptr;
    if (scheme->precision != XFG_FP64 && scheme->precision != XFG_MIXED)
        return efail(-1, "ensemble precision must be XFG_FP64 or XFG_MIXED%s");
    if (scheme->positivity != 0 && scheme->positivity != 1) return efail(-1, "positivity must be 0 or 1%s");
    if (scheme->viscous < 0 || scheme->viscous > 7 || (scheme->viscous && !(scheme->viscous & 1)))
        return efail(-1, "viscous must be Visc | Visc_Heat << 1 | Visc_Diffu << 2%s");
    if (scheme->viscous && !scheme->cop)
        return efail(-1, "viscous fluxes need a mixture (cop = 1): the single-gas states compute no temperature%s");
    if (scheme->scheme_order < 5 || scheme->scheme_order > 7) return efail(-1, "scheme_order must be 5, 6 or 7%s");
    const int ns = scheme->cop ? scheme->num_species : 1;
    if (scheme->cop && (!thermal || thermal->num_species != ns))
        return efail(-1, "a mixture ensemble needs the thermal tables of its num_species%s");
    // mixtures with the positivity limiter keep the uncontracted face sweeps in the FP64 form, as
    // the single-grid path does (its theta amplifies the rounding of the high-order flux)
    const int table_prec = scheme->cop && scheme->positivity && scheme->precision == XFG_FP64 ? XFG_FP64_STRICT
                                                                                           : scheme->precision;
    const EnsOps *ops = find_ens_ops(scheme->cop ? 1 : 0, ns, table_prec);
    if (!ops || !ops->faces)
        return efail(-1, "no batched kernels for this gas model (single gas, or a mixture of 5 species)%s");
    ECK(cudaSetDevice(device));
    xfg_ensemble *e = new xfg_ensemble();
    e->device = device, e->sc = *scheme, e->capacity = capacity;
    e->ops = ops, e->NS = ns, e->E = scheme->cop ? ns + 4 : 5;
    std::memset(&e->th, 0, sizeof e->th);
    e->th.ncop_gamma = scheme->ncop_gamma;
    e->th.nasa = scheme->cop ? (scheme->thermo ? 1 : 0) : 1;
    if (scheme->cop) {  // the thermo tables as xfg_create passes them to the kernels
        for (int n = 0; n < XFG_MAX_SPECIES; n++) e->th.Ri[n] = thermal->Ri[n], e->th._Wi[n] = thermal->_Wi[n];
        for (int q = 0; q < XFG_MAX_SPECIES * 21; q++) e->th.Hia[q] = thermal->Hia[q];
        for (int q = 0; q < XFG_MAX_SPECIES * 6; q++) e->th.Hib[q] = thermal->Hib[q];
    }
    e->hm.assign(capacity, Member{});
    for (auto &m : e->hm) std::memset(&m, 0, sizeof m);
    e->m_off.assign(capacity, 0), e->m_len.assign(capacity, 0), e->blocks.assign(capacity, xfg_block{});
    cudaError_t err = cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaMalloc(&e->pool, pool_bytes);
    if (err == cudaSuccess) err = cudaMalloc(&e->dm, sizeof(Member) * capacity);
    if (err == cudaSuccess) err = cudaMalloc(&e->doff, sizeof(int) * PH_N * (3 * (size_t)capacity + 1));
    if (err == cudaSuccess) err = cudaMalloc(&e->ddt, sizeof(double) * 8 * capacity);
    if (err == cudaSuccess) err = cudaMalloc(&e->derr, sizeof(int) * 8 * capacity);
    if (err == cudaSuccess) err = cudaMallocHost(&e->hdt, sizeof(double) * 8 * capacity);
    if (err == cudaSuccess) err = cudaMallocHost(&e->herr, sizeof(int) * 8 * capacity);
    if (err == cudaSuccess) err = cudaEventCreate(&e->ev[0]);
    if (err == cudaSuccess) err = cudaEventCreate(&e->ev[1]);
    if (err == cudaSuccess) err = cudaMemsetAsync(e->ddt, 0, sizeof(double) * 8 * capacity, e->st);
    if (err == cudaSuccess) err = cudaMemsetAsync(e->derr, 0, sizeof(int) * 8 * capacity, e->st);
    if (err == cudaSuccess && scheme->cop) {  // the mixed form's scaled enthalpy tables
        std::vector<double> hsc(THERMO_SC_DOUBLES);
        std::vector<char> hb(THERMO_SC_BYTES);
        scaled_thermo_table(e->th, hsc.data());
        std::memcpy(hb.data(), hsc.data(), THERMO_SC_DOUBLES * sizeof(double));
        float *hf = (float *)(hb.data() + THERMO_SC_DOUBLES * sizeof(double));
        for (int q = 0; q < THERMO_SC_DOUBLES; q++) hf[q] = (float)hsc[q];
        err = cudaMalloc(&e->dhsc, THERMO_SC_BYTES);
        if (err == cudaSuccess) err = cudaMemcpyAsync(e->dhsc, hb.data(), THERMO_SC_BYTES, cudaMemcpyHostToDevice, e->st);
        e->th.hsc = e->dhsc;
        e->th.hscf = (const float *)(e->dhsc + THERMO_SC_DOUBLES);
    }
    if (err == cudaSuccess && scheme->viscous) {  // transport tables, filled by xfg_ensemble_set_transport
        const int ns = e->NS;
        const size_t nd = 8 * ns + 2 * ns * ns + ns, nf = 8 * ns + 2 * ns * ns;
        err = cudaMalloc(&e->dtr, nd * sizeof(double) + nf * sizeof(float));
        if (err == cudaSuccess) {
            e->dtrf = (float *)(e->dtr + nd);
            err = cudaMemsetAsync(e->dtr, 0, nd * sizeof(double) + nf * sizeof(float), e->st);
        }
    }
    if (err == cudaSuccess) err = cudaStreamSynchronize(e->st);
    if (err != cudaSuccess) {
        xfg_ensemble_destroy(e);
        return efail(-3, "ensemble allocation failed: %s", cudaGetErrorString(err));
    }
    e->pool_bytes = pool_bytes;
    e->alloc.init(pool_bytes);
    e->fused_ok = !scheme->cop && scheme->precision == XFG_MIXED && scheme->scheme_order == 5 && !scheme->positivity &&
                  (scheme->artificial_type == XFG_LLF || scheme->artificial_type == XFG_ROE);
    if (e->fused_ok) {
        const double gm1 = scheme->ncop_gamma - 1.0;
        e->fk.gamma = (float)scheme->ncop_gamma;
        e->fk.gm1h = (float)gm1;
        e->fk.gm1l = (float)(gm1 - (double)e->fk.gm1h);
        e->fk.igm1 = (float)(1.0 / gm1);
        err = cudaFuncSetAttribute(kb_fused<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(FusedTile));
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(kb_fused<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(FusedTile));
        if (err != cudaSuccess) {
            xfg_ensemble_destroy(e);
            return efail(-2, "fused stage set-up failed: %s", cudaGetErrorString(err));
        }
    }
    *out = e;
    return 0;
}

int xfg_ensemble_destroy(xfg_ensemble *e) {
    if (!e) return 0;
    cudaSetDevice(e->device);
    if (e->st) cudaStreamSynchronize(e->st);
    if (e->graph) cudaGraphExecDestroy(e->graph);
    for (auto &v : e->ev)
        if (v) cudaEventDestroy(v);
    cudaFree(e->pool), cudaFree(e->dm), cudaFree(e->doff), cudaFree(e->ddt), cudaFree(e->derr), cudaFree(e->dhsc);
    cudaFree(e->dtr);
    if (e->hdt) cudaFreeHost(e->hdt);
    if (e->herr) cudaFreeHost(e->herr);
    if (e->st) cudaStreamDestroy(e->st);
    delete e;
    return 0;
}

size_t xfg_ensemble_member_bytes(const xfg_block *block, int precision) {
    return block ? member_bytes(*block, 0, 1, precision == XFG_MIXED, 0) : 0;
}

int xfg_ensemble_set_transport(xfg_ensemble *e, const xfg_transport *tr) {
    if (!e || !tr) return efail(-1, "null argument%s");
    if (!e->sc.viscous) return efail(-1, "the scheme has no viscous fluxes (xfg_scheme.viscous = 0)%s");
    std::vector<double> t;
    std::vector<float> tf;
    if (int rc = pack_transport(tr, e->NS, t, tf)) return rc;
    ECK(cudaSetDevice(e->device));
    ECK(cudaMemcpyAsync(e->dtr, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice, e->st));
    ECK(cudaMemcpyAsync(e->dtrf, tf.data(), tf.size() * sizeof(float), cudaMemcpyHostToDevice, e->st));
    ECK(cudaStreamSynchronize(e->st));
    e->transport_ready = true;
    return 0;
}

size_t xfg_ensemble_member_bytes_for(const xfg_block *block, const xfg_scheme *scheme) {
    if (!block || !scheme) return 0;
    return member_bytes(*block, scheme->cop ? 1 : 0, scheme->cop ? scheme->num_species : 1,
                        scheme->precision == XFG_MIXED, scheme->cop ? scheme->viscous : 0);
}

int xfg_ensemble_add(xfg_ensemble *e, const xfg_block *block, const double *U_aos, double target_t, int *slot) {
    return xfg_ensemble_add_t(e, block, U_aos, nullptr, target_t, slot);
}

int xfg_ensemble_add_t(xfg_ensemble *e, const xfg_block *block, const double *U_aos, const double *T, double target_t,
                       int *slot) {
    if (!e || !block || !U_aos || !slot) return efail(-1, "null argument%s");
    if (e->sc.cop && !T) return efail(-1, "a mixture member needs its temperature (the Newton warm start)%s");
    *slot = -1;
    int s = -1;
    for (int q = 0; q < e->capacity; q++)
        if (!e->hm[q].active && e->m_len[q] == 0) { s = q; break; }
    if (s < 0) return 1;  // no free slot
    const bool mixed = e->sc.precision == XFG_MIXED;
    const size_t need = member_bytes(*block, e->sc.cop, e->NS, mixed, e->sc.viscous);
    size_t off = 0;
    if (!e->alloc.alloc(need, &off)) return 2;  // no memory: admission waits
    ECK(cudaSetDevice(e->device));
    Member &m = e->hm[s];
    std::memset(&m, 0, sizeof m);
    carve(m, e->pool + off, *block, e->sc.cop, e->NS, mixed, e->sc.viscous, e->dtr, e->dtrf);
    m.f.dtbuf = e->ddt + 8 * s;
    m.f.err = e->derr + 8 * s;
    m.active = 1;
    m.fused = e->fused_ok && two_d(*block) ? 1 : 0;
    e->m_off[s] = off, e->m_len[s] = need, e->blocks[s] = *block;
    const long long N = m.g.ncell(), P = m.g.pitch;
    const int E = e->E;
    ECK(cudaMemsetAsync(e->pool + off, 0, need, e->st));
    double *stage = m.f.LU;  // AoS staging in LU (E * P >= E * N)
    ECK(cudaMemcpyAsync(stage, U_aos, sizeof(double) * E * N, cudaMemcpyDefault, e->st));
    kb_aos_to_soa<<<(unsigned)((E * N + 255) / 256), 256, 0, e->st>>>(stage, m.f.U, E, N, P);
    ECK(cudaMemcpyAsync(m.f.U1, m.f.U, sizeof(double) * E * P, cudaMemcpyDeviceToDevice, e->st));
    if (T) ECK(cudaMemcpyAsync(m.f.T, T, sizeof(double) * N, cudaMemcpyDefault, e->st));
    if (m.fused)  // the first stage's output buffer starts as U1 does (ghost cells of no-op sides)
        ECK(cudaMemcpyAsync(m.f.U2, m.f.U, sizeof(double) * 5 * P, cudaMemcpyDeviceToDevice, e->st));
    double dtb[8] = {0.0, 0.0, target_t, 0.0, 0.0, 0.0, 0.0, 0.0};
    ECK(cudaMemcpyAsync(m.f.dtbuf, dtb, sizeof dtb, cudaMemcpyHostToDevice, e->st));
    ECK(cudaMemsetAsync(m.f.err, 0, 8 * sizeof(int), e->st));
    // main.cpp:45-47 for this member: BoundaryCondition(U) and UpdateStates(U) (dt maxima on)
    LaunchCtx c;
    std::memset(&c, 0, sizeof c);
    c.g = m.g, c.f = m.f, c.th = e->th, c.st = e->st, c.artificial = e->sc.artificial_type;
    c.ghost = e->sc.ghost_species;
    for (int q = 0; q < 6; q++) c.bc[q] = m.bc[q];
    c.precision = e->sc.precision;
    const Ops *ops = find_ops(e->sc.cop ? 1 : 0, e->NS, e->sc.scheme_order, e->sc.precision);
    if (!ops) return efail(-1, "no single-grid kernels for this scheme%s");
    ops->bc(c, m.f.U, nullptr);
    ops->states(c, m.f.U, 1, 0);
    ECK(cudaGetLastError());
    ECK(cudaStreamSynchronize(e->st));
    e->dirty = true;
    *slot = s;
    return 0;
}

int xfg_ensemble_remove(xfg_ensemble *e, int slot) {
    if (!e || slot < 0 || slot >= e->capacity || e->m_len[slot] == 0) return efail(-1, "bad slot%s");
    ECK(cudaStreamSynchronize(e->st));
    e->alloc.release(e->m_off[slot], e->m_len[slot]);
    e->m_len[slot] = 0, e->m_off[slot] = 0;
    std::memset(&e->hm[slot], 0, sizeof(Member));
    e->dirty = true;
    return 0;
}

int xfg_ensemble_advance(xfg_ensemble *e, int nsteps, int use_graph, float *device_ms) {
    if (!e) return efail(-1, "null ensemble%s");
    if (e->sc.viscous && !e->transport_ready) return efail(-1, "viscous scheme: call xfg_ensemble_set_transport first%s");
    ECK(cudaSetDevice(e->device));
    if (e->dirty) {
        int rc = rebuild(e);
        if (rc) return rc;
    }
    if (e->order.empty()) return 0;
    const int G = use_graph ? e->graph_steps : 1;
    if (use_graph && (!e->graph || e->graph_built_steps != G)) {
        if (e->graph) cudaGraphExecDestroy(e->graph), e->graph = nullptr;
        cudaGraph_t g;
        ECK(cudaStreamBeginCapture(e->st, cudaStreamCaptureModeThreadLocal));
        for (int q = 0; q < G; q++) launch_step(e);
        cudaError_t err = cudaStreamEndCapture(e->st, &g);
        if (err != cudaSuccess) return efail(-2, "graph capture failed: %s", cudaGetErrorString(err));
        err = cudaGraphInstantiate(&e->graph, g, 0);
        cudaGraphDestroy(g);
        if (err != cudaSuccess) return efail(-2, "graph instantiate failed: %s", cudaGetErrorString(err));
        e->graph_built_steps = G;
    }
    ECK(cudaEventRecord(e->ev[0], e->st));
    int left = nsteps;
    if (use_graph)
        for (; left >= G; left -= G) ECK(cudaGraphLaunch(e->graph, e->st));
    for (; left > 0; left--) launch_step(e);
    ECK(cudaEventRecord(e->ev[1], e->st));
    ECK(cudaMemcpyAsync(e->hdt, e->ddt, sizeof(double) * 8 * e->capacity, cudaMemcpyDeviceToHost, e->st));
    ECK(cudaMemcpyAsync(e->herr, e->derr, sizeof(int) * 8 * e->capacity, cudaMemcpyDeviceToHost, e->st));
    ECK(cudaStreamSynchronize(e->st));
    ECK(cudaGetLastError());
    if (device_ms) cudaEventElapsedTime(device_ms, e->ev[0], e->ev[1]);
    int rc = 0;
    for (int s : e->order)
        if (e->herr[8 * s + ERR_STATE]) rc = 10000;
        else if (e->herr[8 * s + ERR_PRIM] && !rc) rc = 1;
    return rc;
}

// Time, steps, done flag and error of a member as of the last xfg_ensemble_advance.
int xfg_ensemble_status(xfg_ensemble *e, int slot, double *t, int *steps, int *done) {
    if (!e || slot < 0 || slot >= e->capacity) return efail(-1, "bad slot%s");
    const double *b = e->hdt + 8 * slot;
    if (t) *t = b[1];
    if (steps) *steps = (int)b[3];
    if (done) *done = b[4] != 0.0;
    if (e->herr[8 * slot + ERR_STATE]) return 10000;
    return e->herr[8 * slot + ERR_PRIM] ? 1 : 0;
}

int xfg_ensemble_get_state(xfg_ensemble *e, int slot, double *U_aos) {
    if (!e || slot < 0 || slot >= e->capacity || e->m_len[slot] == 0 || !U_aos) return efail(-1, "bad slot%s");
    ECK(cudaSetDevice(e->device));
    const Member &m = e->hm[slot];
    const long long N = m.g.ncell(), P = m.g.pitch;
    const int E = e->E;
    kb_soa_to_aos<<<(unsigned)((E * N + 255) / 256), 256, 0, e->st>>>(m.f.U, m.f.LU, E, N, P);
    ECK(cudaMemcpyAsync(U_aos, m.f.LU, sizeof(double) * E * N, cudaMemcpyDefault, e->st));
    ECK(cudaStreamSynchronize(e->st));
    return 0;
}

int xfg_ensemble_get_option(xfg_ensemble *e, int option, int *value) {
    if (!e || !value) return efail(-1, "null argument%s");
    if (option == XFG_ENS_LARGEST_FIRST) *value = e->largest_first;
    else if (option == XFG_ENS_FUSED_FACES) *value = e->fused_faces;
    else if (option == XFG_ENS_GRAPH_STEPS) *value = e->graph_steps;
    else if (option >= XFG_ENS_TILE_1D && option <= XFG_ENS_TILE_3D) *value = e->ltx[option - XFG_ENS_TILE_1D];
    else return efail(-1, "unknown option%s");
    return 0;
}

// A member as a checkpoint file of the reference's format (XFLUIDS::Output_Ubak,
// src/XFLUIDS.cpp:658-687): its step count, time and U.
int xfg_ensemble_checkpoint_write(xfg_ensemble *e, int slot, const char *path, float duration, double *lam_out) {
    if (!e || !path || slot < 0 || slot >= e->capacity || e->m_len[slot] == 0) return efail(-1, "bad slot%s");
    const Member &m = e->hm[slot];
    std::vector<double> U((size_t)m.g.ncell() * e->E);
    int rc = xfg_ensemble_get_state(e, slot, U.data());
    if (rc) return rc;
    double b[8];
    ECK(cudaMemcpy(b, m.f.dtbuf, sizeof b, cudaMemcpyDeviceToHost));
    if (lam_out) {  // the GetDt maxima the member's next step will use
        unsigned long long lam[3];
        ECK(cudaMemcpy(lam, m.f.lam, sizeof lam, cudaMemcpyDeviceToHost));
        for (int q = 0; q < 3; q++) std::memcpy(&lam_out[q], &lam[q], 8);
    }
    const int step = (int)b[3];
    const double time = b[1];
    std::FILE *fp = std::fopen(path, "wb");
    if (!fp) return efail(-1, "cannot open %s for writing", path);
    bool ok = std::fwrite(&step, sizeof step, 1, fp) == 1 && std::fwrite(&time, sizeof time, 1, fp) == 1 &&
              std::fwrite(&duration, sizeof duration, 1, fp) == 1 &&
              std::fwrite(U.data(), sizeof(double), U.size(), fp) == U.size();
    ok = (std::fclose(fp) == 0) && ok;
    return ok ? 0 : efail(-1, "write of %s failed", path);
}

// Admit a member from a checkpoint file (XFLUIDS::Read_Ubak, src/XFLUIDS.cpp:689-724): U, time and
// step count as saved, then the member's BoundaryCondition + UpdateStates as xfg_ensemble_add.
int xfg_ensemble_add_checkpoint(xfg_ensemble *e, const xfg_block *block, const char *path, double target_t,
                                const double *lam_in, int *slot) {
    if (!e || !block || !path || !slot) return efail(-1, "null argument%s");
    *slot = -1;
    if (e->sc.cop) return efail(-1, "a mixture member cannot be restored from a checkpoint (it holds no temperature)%s");
    const size_t n = (size_t)block->Xmax * block->Ymax * block->Zmax * 5;
    std::FILE *fp = std::fopen(path, "rb");
    if (!fp) return efail(-1, "cannot open %s", path);
    int step = 0;
    double time = 0.0;
    float dur = 0.f;
    std::vector<double> U(n);
    bool ok = std::fread(&step, sizeof step, 1, fp) == 1 && std::fread(&time, sizeof time, 1, fp) == 1 &&
              std::fread(&dur, sizeof dur, 1, fp) == 1 && std::fread(U.data(), sizeof(double), n, fp) == n;
    const bool extra = ok && std::fgetc(fp) != EOF;
    std::fclose(fp);
    if (!ok || extra) return efail(-1, "%s is not a checkpoint of this block", path);
    int rc = xfg_ensemble_add(e, block, U.data(), target_t, slot);
    if (rc) return rc;  // 1 / 2: no slot or no memory, nothing admitted
    const Member &m = e->hm[*slot];
    const double tb[4] = {0.0, time, target_t, (double)step};
    ECK(cudaMemcpy(m.f.dtbuf, tb, sizeof tb, cudaMemcpyHostToDevice));
    if (lam_in) {  // continue with the dt the saved run would have taken next
        unsigned long long lam[3];
        for (int q = 0; q < 3; q++) std::memcpy(&lam[q], &lam_in[q], 8);
        ECK(cudaMemcpy(m.f.lam, lam, sizeof lam, cudaMemcpyHostToDevice));
    }
    return 0;
}

int xfg_ensemble_set_option(xfg_ensemble *e, int option, int value) {
    if (!e) return efail(-1, "null ensemble%s");
    if (option == XFG_ENS_LARGEST_FIRST) e->largest_first = value ? 1 : 0;
    else if (option == XFG_ENS_FUSED_FACES) e->fused_faces = value ? 1 : 0;
    else if (option == XFG_ENS_GRAPH_STEPS) {
        if (value < 1 || value > 64) return efail(-1, "graph steps must be in 1..64%s");
        e->graph_steps = value;
        return 0;  // the graph is re-captured at the next advance
    } else if (option >= XFG_ENS_TILE_1D && option <= XFG_ENS_TILE_3D) {
        if (value < 3 || value > 7) return efail(-1, "face tile: log2 of its x extent must be in 3..7%s");
        e->ltx[option - XFG_ENS_TILE_1D] = value;
    } else
        return efail(-1, "unknown option%s");
    e->dirty = true;
    return 0;
}

size_t xfg_ensemble_free_bytes(xfg_ensemble *e) { return e ? e->alloc.free_bytes() : 0; }

int xfg_ensemble_active(xfg_ensemble *e) {
    if (!e) return 0;
    int n = 0;
    for (auto &m : e->hm) n += m.active ? 1 : 0;
    return n;
}

}  // extern "C"
