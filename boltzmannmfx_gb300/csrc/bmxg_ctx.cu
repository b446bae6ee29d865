// bmxg_ctx.cu -- host side of the C ABI (include/bmxg.h): context lifetime,
// state upload / readback, the graph-captured step loop, neighbour-list
// export, statistics and the launch-shape autotuner.
//
// Stands behind BMXParticleContainer::EvolveParticles
// (src/des/bmx_pc.H:126-129, src/des/bmx_pc_interaction.cpp:13-495).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../../include/bmxg.h"
#include "bmxg_kernels.cuh"

using namespace bmxg;

namespace {

struct GraphKey {
    double dt;
    int precision;
    int parity;
    int single;  // -1: kResyncEvery steps; 0 / 1: one step without / with the FP32F re-sync
    bool operator<(const GraphKey &o) const
    {
        if (dt != o.dt) return dt < o.dt;
        if (precision != o.precision) return precision < o.precision;
        if (parity != o.parity) return parity < o.parity;
        return single < o.single;
    }
};

struct Shape {
    int block = 256;
    int grid = 0;  // 0: derive from occupancy
};

}  // namespace

struct bmxg_ctx {
    std::string err;
    bmxg_params prm{};
    int ncol = 0;
    std::vector<bmxg_geometry> geoms;
    int device = 0;
    int nsm = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    // device allocations
    std::vector<void *> allocs;
    DevState S{};
    DevGeom *d_geoms = nullptr;
    int *d_cbase = nullptr;                 // ncol + 1 colony slot offsets (device)
    std::vector<int> h_cbase;
    std::vector<DevGeom> h_geoms;
    DevCounters *d_cnt = nullptr;
    DevCounters *h_cnt = nullptr;  // pinned
    int *scan_scratch = nullptr;
    // staging in caller order
    double *ud = nullptr;  // n doubles
    int *ui = nullptr;     // 13 n ints
    int *uperm = nullptr;

    int64_t n = 0;
    bool have_state = false;
    bool stepped = false;
    int parity = 0;
    std::vector<int64_t> offsets;

    std::map<GraphKey, cudaGraphExec_t> graphs;
    std::map<GraphKey, int> graph_kernels;  // kernels per replay of each graph
    Shape sh_sphere[2], sh_rod, sh_misc;
    // list path shapes (bmxg_autotune): k_list_step's block and passes per
    // chunk (0: the launcher's rule), k_list_build's block
    int ls_block = kListStepBlock, ls_passes = 0, lb_block = kListBuildBlock;
    bool ls_persist = false;  // the list step as one wave of blocks taking chunks from a counter
    bmxg_stats stats{};
    int64_t launches = 0;                   // kernels enqueued (graph nodes counted per replay)
    bool profiling = false;
    std::vector<cudaEvent_t> kev;           // event pairs around the force kernel, profiling mode
    size_t kev_used = 0;

    // differentiation form
    double ext_gamma = 0.0, ext_mu = 0.0;
    double *d_adh = nullptr;                // per-slot adhesion in use (nullptr: zero)
    double *adh_buf = nullptr;              // its buffer, allocated with the state
    std::vector<void *> dallocs;            // adjoint buffers (freed with the state)
    double *ckpt = nullptr;                 // (nseg + 1) x 3n positions, slot order
    double *segbuf = nullptr;               // ckpt_every x 3n positions of one segment
    double *lam[2] = {nullptr, nullptr};    // adjoint of the positions, 3 planes
    double *gacc = nullptr, *gadh = nullptr, *gout = nullptr, *xT = nullptr;
    int traj_T = -1, traj_k = 0;
    double traj_dt = 0.0;

    bool vel32 = false;       // the last step's velocities are in the FP32F buffers
    bool vel64_zero = false;  // the FP64 velocity planes (vx .. wz) hold zeros: a load zeroed them
                              // and no kernel that writes them ran since
    int64_t step_count = 0;   // steps since set_state (FP32F re-sync schedule)

    // FP32F neighbour list with a skin (k_list.cu)
    int list_mode = 1;            // 1: FP32F sphere steps use the list where it is exact; 0: never
    bool list_on = false;         // the steps being enqueued use the list
    bool list_valid = false;      // the list and its frozen bins describe the state
    bool bins_exact = true;       // bins of buffer `parity` are the reference's (list steps freeze them)
    double rmax = 0.0;            // largest radius of the state
    int64_t ncells_total = 0;     // 3D cells over all colonies
    int *cell_scratch = nullptr;  // scan scratch of the list build (column counts, group entries)
    float skin_cur = 0.0f;        // skin of the list control block
    ListCtl *h_lctl = nullptr;    // pinned copy of the control block
    unsigned long long body_runs_seen = 0;  // list builds already counted as launches
    bool capturing = false;       // enqueue_step runs inside a graph capture
    bool pair_capture = false;    // list steps record their gated pairs (S.pcap)
    bool pcap_valid = false;      // S.pcap holds the last step's gated pairs
    bool fx_ahead = false;        // list steps moved the fixed-point positions past the FP64 ones
    std::vector<FxGeom> h_fxg;    // per colony fixed-point geometry of the list path
    FxGeom *d_fxg = nullptr;
    cudaStream_t body_stream = nullptr;     // captures the bodies of conditional nodes

    // loads and stores of host arrays: the copies run on io_stream, overlapped
    // with the sort, gather and scatter kernels on `stream`; the device
    // staging is kept (and grown) across calls
    cudaStream_t io_stream = nullptr;
    cudaEvent_t io_ev[8] = {};
    char *io_buf = nullptr;
    size_t io_cap = 0;
    unsigned long long *d_chk = nullptr;    // state-check flags (4), device
    unsigned long long *h_chk = nullptr;    // and pinned host
};

namespace {

int sync_fp64(bmxg_ctx *ctx);

int fail(bmxg_ctx *c, int code, const std::string &msg)
{
    if (c) c->err = msg;
    return code;
}

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? BMXG_ERR_OOM : BMXG_ERR_CUDA,  \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                  \
    } while (0)

// Enqueue a launcher (it returns how many kernels it launched), count them,
// and turn a launch error into a status naming the launcher.
#define LAUNCH(call)                                                                             \
    do {                                                                                         \
        ctx->launches += (call);                                                                 \
        cudaError_t e_ = cudaPeekAtLastError();                                                  \
        if (e_ != cudaSuccess)                                                                   \
            return fail(ctx, BMXG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <class T>
int dalloc(bmxg_ctx *ctx, T **p, size_t count)
{
    void *q = nullptr;
    if (count == 0) count = 1;
    CK(cudaMalloc(&q, count * sizeof(T)));
    ctx->allocs.push_back(q);
    *p = (T *)q;
    return BMXG_OK;
}

void drop_graphs(bmxg_ctx *ctx)
{
    for (auto &g : ctx->graphs) cudaGraphExecDestroy(g.second);
    ctx->graphs.clear();
    ctx->graph_kernels.clear();
}

void free_adjoint(bmxg_ctx *ctx)
{
    for (void *p : ctx->dallocs) cudaFree(p);
    ctx->dallocs.clear();
    ctx->ckpt = ctx->segbuf = ctx->gacc = ctx->gadh = ctx->gout = ctx->xT = nullptr;
    ctx->lam[0] = ctx->lam[1] = nullptr;
    ctx->traj_T = -1;
}

// Device staging of at least `bytes` for host loads and stores.
int ensure_io(bmxg_ctx *ctx, size_t bytes)
{
    if (bytes <= ctx->io_cap) return BMXG_OK;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaStreamSynchronize(ctx->io_stream));
    if (ctx->io_buf) cudaFree(ctx->io_buf);
    ctx->io_buf = nullptr;
    ctx->io_cap = 0;
    CK(cudaMalloc(&ctx->io_buf, bytes));
    ctx->io_cap = bytes;
    return BMXG_OK;
}

// Waits for the load / store copies still reading or writing caller memory
// when a call returns early.
struct JoinIo {
    cudaStream_t s;
    ~JoinIo()
    {
        if (s) cudaStreamSynchronize(s);
    }
};

void free_state(bmxg_ctx *ctx)
{
    drop_graphs(ctx);
    free_adjoint(ctx);
    ctx->d_adh = ctx->adh_buf = nullptr;  // lives in allocs
    for (void *p : ctx->allocs) cudaFree(p);
    ctx->allocs.clear();
    ctx->S = DevState{};
    ctx->d_geoms = nullptr;
    ctx->d_cbase = nullptr;
    ctx->scan_scratch = nullptr;
    ctx->cell_scratch = nullptr;
    ctx->ud = nullptr;
    ctx->ui = nullptr;
    ctx->uperm = nullptr;
    ctx->have_state = false;
    ctx->list_valid = false;
    ctx->fx_ahead = false;
    ctx->d_fxg = nullptr;
    ctx->bins_exact = true;
}

int grid_for(bmxg_ctx *ctx, const Shape &s, int64_t n)
{
    int g = s.grid;
    if (g <= 0) g = ctx->nsm * std::max(1, 2048 / s.block);
    int64_t need = (n + s.block - 1) / s.block;
    if (need < 1) need = 1;
    return (int)std::min<int64_t>(g, need);
}

// Launch shape of the per-slot stencil kernels (spheres, the differentiation
// form): an autotuned shape when there is one; else one slot per thread in
// 64-thread blocks.  The stencil walks differ in length from slot to slot, and
// small blocks on a grid of every slot let the block scheduler balance them
// (2.73 M spheres: FP64 6.66 -> 5.94 ms, FP32F 657 -> 600 us per step, against
// 256-thread blocks striding over one wave).
void stencil_shape(bmxg_ctx *ctx, const Shape &s, int64_t n, int *grid, int *block)
{
    if (s.grid > 0) {
        *block = s.block;
        *grid = grid_for(ctx, s, n);
    } else {
        *block = kSphereBlock;
        *grid = (int)std::max<int64_t>(1, (n + kSphereBlock - 1) / kSphereBlock);
    }
}

DevParams dev_params(const bmxg_params &p)
{
    DevParams d{p.bndry_width, p.stiffness,     p.z_wall,      p.z_bndry_width, p.z_stiffness,
                p.z_gravity,   p.bond_strength, p.bond_cutoff, p.viscosity,     p.neighborhood};
    d.bw32 = (float)d.bw;
    d.k32 = (float)d.k;
    d.z_k32 = (float)d.z_k;
    d.z_bw32 = (float)d.z_bw;
    d.z_g32 = (float)d.z_g;
    return d;
}

int check_params(const bmxg_params *p)
{
    if (!p) return BMXG_ERR_ARG;
    const double v[10] = {p->bndry_width, p->stiffness,     p->z_wall,      p->z_bndry_width, p->z_stiffness,
                          p->z_gravity,   p->bond_strength, p->bond_cutoff, p->viscosity,     p->neighborhood};
    for (double x : v)
        if (!std::isfinite(x)) return BMXG_ERR_ARG;
    return BMXG_OK;
}

int check_geom(const bmxg_geometry &g, std::string &why)
{
    for (int d = 0; d < 3; ++d) {
        if (!(g.prob_hi[d] > g.prob_lo[d]) || !std::isfinite(g.prob_lo[d]) || !std::isfinite(g.prob_hi[d])) {
            why = "prob_hi must exceed prob_lo";
            return BMXG_ERR_ARG;
        }
        if (g.n_cell[d] < 1 || g.n_cell[d] > (1 << 20)) {
            why = "n_cell out of range";
            return BMXG_ERR_ARG;
        }
        if (g.is_periodic[d] && g.n_cell[d] < 3) {
            why = "a periodic direction needs n_cell >= 3";
            return BMXG_ERR_UNSUPPORTED;
        }
    }
    if (g.is_periodic[2]) {
        why = "z must be non-periodic (the growth surface sits in z)";
        return BMXG_ERR_UNSUPPORTED;
    }
    return BMXG_OK;
}

// Device geometry of each colony, with the column and slot numbering.
void build_geoms(bmxg_ctx *ctx)
{
    ctx->h_geoms.resize(ctx->ncol);
    ctx->h_fxg.resize(ctx->ncol);
    int col_base = 0;
    int64_t cell_base = 0;
    for (int c = 0; c < ctx->ncol; ++c) {
        const bmxg_geometry &g = ctx->geoms[c];
        DevGeom &G = ctx->h_geoms[c];
        std::memset(&G, 0, sizeof(G));
        double diag2 = 0.0;
        for (int d = 0; d < 3; ++d) {
            G.plo[d] = g.prob_lo[d];
            G.phi[d] = g.prob_hi[d];
            G.len[d] = g.prob_hi[d] - g.prob_lo[d];
            G.n[d] = g.n_cell[d];
            G.dx[d] = G.len[d] / (double)G.n[d];
            G.dxi[d] = 1.0 / G.dx[d];
            G.dxf[d] = (float)G.dx[d];
            G.plof[d] = (float)G.plo[d];
            G.dxif[d] = (float)G.dxi[d];
            G.phif[d] = (float)G.phi[d];
            // corners as the device computes them: a product, then a sum, each
            // rounded (volatile keeps the host compiler from fusing them)
            G.ncorner[d] = std::min(G.n[d], kCornerTable);
            for (int bi = 1; bi <= G.ncorner[d]; ++bi) {
                volatile double t = (double)(bi - 1) * G.dx[d];
                G.corner[d][bi - 1] = G.plo[d] + t;
            }
            G.per[d] = g.is_periodic[d] ? 1 : 0;
            diag2 += 4.0 * G.dx[d] * G.dx[d];
        }
        G.col_base = col_base;
        col_base += G.n[0] * G.n[1];
        G.cell_base = (int)std::min<int64_t>(cell_base, INT32_MAX);
        cell_base += (int64_t)G.n[0] * G.n[1] * G.n[2];
        G.slot_base = (int)ctx->offsets[c];
        G.slot_end = (int)ctx->offsets[c + 1];
        // two bins apart at most per axis: |r|^2 < 4 (dx^2 + dy^2 + dz^2)
        G.nbh_trivial = (ctx->prm.neighborhood >= diag2 * (1.0 + 1e-9)) ? 1 : 0;
        G.invny = 1.0f / (float)G.n[1];
        // 64-bit fixed point of the list path: a periodic axis spans the
        // domain, a closed one four lengths from one length below plo
        FxGeom &F = ctx->h_fxg[c];
        std::memset(&F, 0, sizeof(F));
        for (int d = 0; d < 3; ++d) {
            const double span = G.per[d] ? G.len[d] : 4.0 * G.len[d];
            F.o[d] = G.per[d] ? G.plo[d] : G.plo[d] - G.len[d];
            F.u[d] = std::ldexp(span, -64);
            F.uh[d] = (float)std::ldexp(span, -32);
            const long double cx = std::ldexp(1.0L / (long double)span, 64);
            F.c[d] = (float)cx;
            F.cl[d] = (float)(cx - (long double)F.c[d]);
            F.n[d] = G.n[d];
            F.per[d] = G.per[d];
            F.plo[d] = G.plo[d];
            F.phi[d] = G.phi[d];
            F.ozero[d] = F.o[d] == 0.0 ? 1 : 0;
            int k = 0;
            const double fr = std::frexp(span, &k);  // span = fr 2^k, fr in [0.5, 1)
            F.ms[d] = (unsigned long long)std::ldexp(fr, 53);
            F.es[d] = k - 53;
            // 2^64 / span = 2^(64 - es) / ms: q = 2^127 / ms, normalised to 64 bits
            const unsigned __int128 q = ((unsigned __int128)1 << 127) / F.ms[d];
            int bl = 0;
            for (unsigned __int128 v = q; v; v >>= 1) ++bl;
            const int sh = bl - 64;
            F.mc[d] = (unsigned long long)(q >> sh);
            F.ec[d] = (64 - F.es[d]) - 127 + sh;
        }
        {
            const long double t = ((long double)ctx->prm.z_wall - (long double)F.o[2]) / (long double)F.u[2];
            const long double hi = std::floor(t / 4294967296.0L);
            F.zw = (hi <= 0.0L) ? 0u : (hi >= 4294967295.0L ? 4294967295u : (unsigned)hi);
        }
        // height of each z-bin's lower face above the growth surface, with the
        // same FP64 face the re-binning uses, split into a float pair
        G.nwz = std::min(G.n[2] + 2, kWallTable);
        for (int bz = 0; bz < G.nwz; ++bz) {
            const double face = G.plo[2] + (double)(bz - 1) * G.dx[2];
            const double h = face - ctx->prm.z_wall;
            const float hi = (float)h;
            G.wz[bz] = make_float2(hi, (float)(h - (double)hi));
        }
    }
    ctx->ncells_total = cell_base;
}

}  // namespace

extern "C" {

int bmxg_version(void) { return BMXG_ABI_VERSION; }

const char *bmxg_last_error(const bmxg_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int bmxg_create(const bmxg_params *params, int32_t ncolonies, const bmxg_geometry *geoms, bmxg_ctx **out)
{
    if (!out) return BMXG_ERR_ARG;
    *out = nullptr;
    if (check_params(params) || ncolonies < 1 || !geoms) return BMXG_ERR_ARG;
    bmxg_ctx *ctx = new bmxg_ctx();
    ctx->prm = *params;
    ctx->ncol = ncolonies;
    ctx->geoms.assign(geoms, geoms + ncolonies);
    for (int c = 0; c < ncolonies; ++c) {
        std::string why;
        int rc = check_geom(ctx->geoms[c], why);
        if (rc) {
            delete ctx;
            return rc;
        }
    }
    int64_t cols = 0;
    for (auto &g : ctx->geoms) cols += (int64_t)g.n_cell[0] * g.n_cell[1];
    if (cols >= (1LL << 31) - 2) {
        delete ctx;
        return BMXG_ERR_UNSUPPORTED;
    }
    cudaError_t e = cudaGetDevice(&ctx->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, ctx->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_cnt, sizeof(DevCounters));
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_lctl, sizeof(ListCtl));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->body_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->io_stream, cudaStreamNonBlocking);
    for (cudaEvent_t &ev : ctx->io_ev)
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_chk, 4 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_chk, 4 * sizeof(unsigned long long));
    if (e != cudaSuccess) {
        ctx->err = cudaGetErrorString(e);
        bmxg_destroy(ctx);
        return BMXG_ERR_CUDA;
    }
    ctx->stream = ctx->own_stream;
    ctx->sh_sphere[0].block = 256;
    ctx->sh_sphere[1].block = 256;
    ctx->sh_rod.block = 32;  // rod walks: one warp per block balances best (FP64 890 -> 844 us, 50 k segments)
    ctx->sh_misc.block = 256;
    *out = ctx;
    return BMXG_OK;
}

void bmxg_destroy(bmxg_ctx *ctx)
{
    if (!ctx) return;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    free_state(ctx);
    if (ctx->h_cnt) cudaFreeHost(ctx->h_cnt);
    if (ctx->h_lctl) cudaFreeHost(ctx->h_lctl);
    if (ctx->body_stream) cudaStreamDestroy(ctx->body_stream);
    if (ctx->io_stream) {
        cudaStreamSynchronize(ctx->io_stream);
        cudaStreamDestroy(ctx->io_stream);
    }
    for (cudaEvent_t ev : ctx->io_ev)
        if (ev) cudaEventDestroy(ev);
    if (ctx->io_buf) cudaFree(ctx->io_buf);
    if (ctx->d_chk) cudaFree(ctx->d_chk);
    if (ctx->h_chk) cudaFreeHost(ctx->h_chk);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    for (cudaEvent_t e : ctx->kev) cudaEventDestroy(e);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

int bmxg_set_params(bmxg_ctx *ctx, const bmxg_params *params)
{
    if (!ctx) return BMXG_ERR_ARG;
    if (check_params(params)) return fail(ctx, BMXG_ERR_ARG, "non-finite force parameter");
    if (int rc = sync_fp64(ctx)) return rc;  // the list's fixed point restarts from the FP64 positions
    ctx->prm = *params;
    drop_graphs(ctx);
    ctx->list_valid = false;
    if (ctx->have_state) {
        build_geoms(ctx);
        CK(cudaMemcpyAsync(ctx->d_geoms, ctx->h_geoms.data(), sizeof(DevGeom) * ctx->ncol,
                           cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(ctx->d_fxg, ctx->h_fxg.data(), sizeof(FxGeom) * ctx->ncol, cudaMemcpyHostToDevice,
                           ctx->stream));
        if (ctx->S.has_rods && ctx->n) {  // the segment mobilities depend on the viscosity
            const int blk = ctx->sh_misc.block, grd = grid_for(ctx, ctx->sh_misc, ctx->n);
            launch_rod_mobility(ctx->S, dev_params(ctx->prm), grd, blk, ctx->stream);
            CK(cudaGetLastError());
        }
        CK(cudaStreamSynchronize(ctx->stream));
    }
    return BMXG_OK;
}

int bmxg_set_stream(bmxg_ctx *ctx, void *stream)
{
    if (!ctx) return BMXG_ERR_ARG;
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->own_stream;
    if (s != ctx->stream) {
        CK(cudaStreamSynchronize(ctx->stream));
        ctx->stream = s;
        drop_graphs(ctx);
    }
    return BMXG_OK;
}

int bmxg_set_state(bmxg_ctx *ctx, const bmxg_particles *p, const int64_t *colony_offsets, int where)
{
    if (!ctx) return BMXG_ERR_ARG;
    (void)cudaGetLastError();  // drop a non-sticky error another library left on this thread
    if (!p || p->n < 0 || !p->x || !p->y || !p->z || !p->radius || !p->cell_type)
        return fail(ctx, BMXG_ERR_ARG, "x, y, z, radius and cell_type are required");
    if (p->n > (1LL << 30)) return fail(ctx, BMXG_ERR_UNSUPPORTED, "more than 2^30 particles");
    if (where != BMXG_HOST && where != BMXG_DEVICE) return fail(ctx, BMXG_ERR_ARG, "bad `where`");
    const int64_t n = p->n;
    std::vector<int64_t> off(ctx->ncol + 1, 0);
    if (ctx->ncol == 1) {
        off[1] = n;
    } else {
        if (!colony_offsets) return fail(ctx, BMXG_ERR_ARG, "colony_offsets required for several colonies");
        for (int c = 0; c <= ctx->ncol; ++c) off[c] = colony_offsets[c];
        if (off[0] != 0 || off[ctx->ncol] != n) return fail(ctx, BMXG_ERR_ARG, "colony_offsets must span 0..n");
        for (int c = 0; c < ctx->ncol; ++c)
            if (off[c + 1] < off[c]) return fail(ctx, BMXG_ERR_ARG, "colony_offsets must not decrease");
    }
    const cudaMemcpyKind kind = (where == BMXG_HOST) ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    // A load of exactly the state the device holds (a caller that stores the
    // state after a step and loads it back unchanged before the next, as a
    // load-step-store loop does) keeps the slot order, the neighbour list and
    // its frozen frames: the loaded positions, radii and cell types are
    // compared bit for bit with the device state first (a state that passed
    // the checks below before).  Only for spheres and when the caller gives no
    // other field (which would overwrite device fields); what any load resets
    // is reset here as well.
    const bool only_required = !p->velx && !p->vely && !p->velz && !p->wx && !p->wy && !p->wz &&
                               !p->c_length && !p->theta && !p->phi && !p->area && !p->bond_scale &&
                               !p->id && !p->cpu && !p->n_bnds && !p->seg_id1 && !p->seg_id2 && !p->site &&
                               !p->position && !p->fuse_tip && !p->fix_site && !p->fuse_flag &&
                               !p->split_flag && !p->new_flag && !p->dltd;
    const bool same_cand = n && only_required && ctx->have_state && ctx->n == n && ctx->offsets == off &&
                           !ctx->S.has_rods;
    // the comparison reads the device's FP64 positions
    if (same_cand) {
        if (int rc = sync_fp64(ctx)) return rc;
    }
    // Positions, radii and cell types: read in place from device arrays; host
    // arrays go to the staging, radii and cell types first on the compute
    // stream (the state checks need them), positions on the copy stream, so
    // that their copy overlaps the checks and the host's decisions below.
    const double *src_x = p->x, *src_y = p->y, *src_z = p->z, *src_r = p->radius;
    const int *src_ct = p->cell_type;
    JoinIo join{nullptr};
    cudaStream_t st0 = ctx->stream, st1 = ctx->io_stream;
    if (n && where == BMXG_HOST) {
        int rc0 = ensure_io(ctx, (size_t)n * 36 + 256);
        if (rc0) return rc0;
        double *bx = (double *)ctx->io_buf, *by = bx + n, *bz = by + n, *br = bz + n;
        int *bct = (int *)(br + n);
        CK(cudaEventRecord(ctx->io_ev[0], st0));  // earlier kernels on st0 are done with the staging
        CK(cudaStreamWaitEvent(st1, ctx->io_ev[0], 0));
        join.s = st1;
        CK(cudaMemcpyAsync(br, p->radius, sizeof(double) * n, kind, st0));
        CK(cudaMemcpyAsync(bct, p->cell_type, sizeof(int) * n, kind, st0));
        CK(cudaMemcpyAsync(bx, p->x, sizeof(double) * n, kind, st1));
        CK(cudaEventRecord(ctx->io_ev[6], st1));
        CK(cudaMemcpyAsync(by, p->y, sizeof(double) * n, kind, st1));
        CK(cudaEventRecord(ctx->io_ev[7], st1));
        CK(cudaMemcpyAsync(bz, p->z, sizeof(double) * n, kind, st1));
        CK(cudaEventRecord(ctx->io_ev[1], st1));
        src_x = bx;
        src_y = by;
        src_z = bz;
        src_r = br;
        src_ct = bct;
    }
    if (same_cand) {
        cudaStream_t st = ctx->stream;
        const int grd = grid_for(ctx, ctx->sh_misc, n), blk = ctx->sh_misc.block;
        const DevState &S = ctx->S;
        CK(cudaMemsetAsync(ctx->d_chk, 0, sizeof(unsigned long long), st));
        if (join.s) {  // each field as its copy lands: only the last comparison follows the copies
            LAUNCH(launch_same_state(S, ctx->parity, nullptr, nullptr, nullptr, src_r, src_ct, ctx->d_chk, grd, blk,
                                     st));
            CK(cudaStreamWaitEvent(st, ctx->io_ev[6], 0));
            LAUNCH(launch_same_state(S, ctx->parity, src_x, nullptr, nullptr, nullptr, nullptr, ctx->d_chk, grd, blk,
                                     st));
            CK(cudaStreamWaitEvent(st, ctx->io_ev[7], 0));
            LAUNCH(launch_same_state(S, ctx->parity, nullptr, src_y, nullptr, nullptr, nullptr, ctx->d_chk, grd, blk,
                                     st));
            CK(cudaStreamWaitEvent(st, ctx->io_ev[1], 0));
            LAUNCH(launch_same_state(S, ctx->parity, nullptr, nullptr, src_z, nullptr, nullptr, ctx->d_chk, grd, blk,
                                     st));
        } else {
            LAUNCH(launch_same_state(S, ctx->parity, src_x, src_y, src_z, src_r, src_ct, ctx->d_chk, grd, blk, st));
        }
        CK(cudaMemcpyAsync(ctx->h_chk, ctx->d_chk, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (ctx->h_chk[0] == 0) {
            // velocities to zero (unless no kernel wrote them since the last
            // load zeroed them) and the counters; stream-ordered before
            // whatever the caller enqueues next
            if (!ctx->vel64_zero)
                for (double *v : {S.vx, S.vy, S.vz, S.wx, S.wy, S.wz})
                    CK(cudaMemsetAsync(v, 0, sizeof(double) * n, st));
            CK(cudaMemsetAsync(ctx->d_cnt, 0, sizeof(DevCounters), st));
            CK(cudaGetLastError());
            ctx->vel64_zero = true;
            ctx->stepped = false;
            ctx->vel32 = false;
            ctx->pcap_valid = false;
            ctx->d_adh = nullptr;
            free_adjoint(ctx);
            std::memset(&ctx->stats, 0, sizeof(ctx->stats));
            ctx->stats.n_particles = n;
            return BMXG_OK;
        }
    }
    ctx->vel64_zero = false;  // (until the full load below has set every plane)
    // cell types decide which path runs (rods need their fields) and the
    // largest radius whether the FP32F list is exact: checked on the device,
    // one small read-back
    bool rods = false;
    double rmax = 0.0;
    if (n) {
        CK(cudaMemsetAsync(ctx->d_chk, 0, 4 * sizeof(unsigned long long), st0));
        Shape sh;
        launch_check_state(src_ct, src_r, (int)n, ctx->d_chk, grid_for(ctx, sh, n), sh.block, st0);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(ctx->h_chk, ctx->d_chk, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st0));
        const cudaError_t e = cudaStreamSynchronize(st0);
        if (e != cudaSuccess) return fail(ctx, BMXG_ERR_CUDA, std::string("state check: ") + cudaGetErrorString(e));
        const unsigned long long *h = ctx->h_chk;
        if (h[0]) return fail(ctx, BMXG_ERR_ARG, "cell_type must be 0 or 1");
        rods = h[1] != 0;
        const uint64_t rb = h[2];
        std::memcpy(&rmax, &rb, sizeof(rmax));
        if (h[3]) rmax = std::nan("");
    }
    if (rods && (!p->c_length || !p->theta || !p->phi || !p->area || !p->id || !p->cpu || !p->n_bnds ||
                 !p->seg_id1 || !p->seg_id2 || !p->site))
        return fail(ctx, BMXG_ERR_ARG, "rod segments need c_length, theta, phi, area, id, cpu and the bond table");

    CK(cudaStreamSynchronize(ctx->stream));
    // Same particle count, colony layout and cell-type mix as the loaded
    // state: keep the device buffers (and the captured step graphs, which
    // only hold their addresses) and overwrite the contents.
    const bool reuse = ctx->have_state && ctx->n == n && ctx->offsets == off && ctx->S.has_rods == (rods ? 1 : 0);
    if (!reuse) free_state(ctx);
    ctx->n = n;
    ctx->offsets = off;
    build_geoms(ctx);
    int64_t ncols = 0;
    for (auto &g : ctx->geoms) ncols += (int64_t)g.n_cell[0] * g.n_cell[1];

    DevState &S = ctx->S;
    S.n = (int)n;
    S.ncol = ctx->ncol;
    S.ncols_total = (int)ncols;
    S.has_rods = rods ? 1 : 0;
    int rc = BMXG_OK;
#define AL(ptr, cnt)                       \
    do {                                   \
        rc = dalloc(ctx, &(ptr), (cnt));   \
        if (rc) return rc;                 \
    } while (0)
    if (!reuse) {
    AL(ctx->d_geoms, ctx->ncol);
    AL(ctx->d_fxg, ctx->ncol);
    AL(ctx->d_cbase, ctx->ncol + 1);
    AL(ctx->d_cnt, 1);
    for (int k = 0; k < 2; ++k) {
        AL(S.x[k], n); AL(S.y[k], n); AL(S.z[k], n);
        AL(S.rel[k], n); AL(S.col[k], n); AL(S.iz[k], n);
        AL(S.perm[k], n); AL(S.colstart[k], ncols + 1);
        AL(S.srel[k], n); AL(S.siz[k], n); AL(S.rank[k], n);
    }
    AL(S.colcnt, ncols); AL(S.tmp, n); AL(S.lkey, n);
    AL(S.rad, n); AL(S.orig, n); AL(S.ctype, n);
    AL(S.vx, n); AL(S.vy, n); AL(S.vz, n); AL(S.wx, n); AL(S.wy, n); AL(S.wz, n);
    AL(S.vxf, n); AL(S.vyf, n); AL(S.vzf, n);
    AL(ctx->scan_scratch, scan_scratch_ints((int)ncols));
    AL(ctx->ud, n); AL(ctx->ui, 13 * n + 1); AL(ctx->uperm, n);
    if (rods) {
        AL(S.clen, n); AL(S.area, n); AL(S.bscale, n);
        for (int k = 0; k < 2; ++k) { AL(S.theta[k], n); AL(S.phi[k], n); AL(S.trig[k], n); AL(S.tab[k], 13 * n); }
        AL(S.id, n); AL(S.cpu, n); AL(S.fuse_tip, n); AL(S.position, n); AL(S.fix_site, n);
        AL(S.fflag, n); AL(S.sflag, n); AL(S.nflag, n); AL(S.dltd, 6 * n); AL(S.fc, 6 * n); AL(S.axf, n); AL(S.mob, n);
    }
    }  // !reuse
#undef AL
    S.geoms = ctx->d_geoms;
    S.fxg = ctx->d_fxg;
    S.cbase = ctx->d_cbase;
    S.cnt = ctx->d_cnt;
    cudaStream_t st = ctx->stream;
    if (!reuse) {  // same colonies as the loaded state: the device copies are current
        CK(cudaMemcpyAsync(ctx->d_geoms, ctx->h_geoms.data(), sizeof(DevGeom) * ctx->ncol, cudaMemcpyHostToDevice,
                           st));
        CK(cudaMemcpyAsync(ctx->d_fxg, ctx->h_fxg.data(), sizeof(FxGeom) * ctx->ncol, cudaMemcpyHostToDevice, st));
        ctx->h_cbase.assign(off.begin(), off.end());
        CK(cudaMemcpyAsync(ctx->d_cbase, ctx->h_cbase.data(), sizeof(int) * (ctx->ncol + 1), cudaMemcpyHostToDevice,
                           st));
    }
    CK(cudaMemsetAsync(ctx->d_cnt, 0, sizeof(DevCounters), st));
    CK(cudaMemsetAsync(S.colcnt, 0, sizeof(int) * std::max<int64_t>(ncols, 1), st));
    if (n == 0) {
        CK(cudaMemsetAsync(S.colstart[0], 0, sizeof(int) * (ncols + 1), st));
        CK(cudaMemsetAsync(S.colstart[1], 0, sizeof(int) * (ncols + 1), st));
        CK(cudaStreamSynchronize(st));
        ctx->have_state = true;
        ctx->parity = 0;
        return BMXG_OK;
    }
    const int blk = ctx->sh_misc.block;
    const int grd = grid_for(ctx, ctx->sh_misc, n);
    if (join.s) CK(cudaStreamWaitEvent(st, ctx->io_ev[1], 0));  // staged positions
    // canonical order of the caller's particles
    LAUNCH(launch_user_bin(S, src_x, src_y, src_z, S.col[1], S.iz[1], grd, blk, st));
    LAUNCH(launch_scan(S.colcnt, S.colstart[1], (int)ncols, ctx->scan_scratch, st));
    LAUNCH(launch_user_scatter_canon(S, S.col[1], S.iz[1], S.colstart[1], ctx->uperm, grd, blk, st));
    // positions, radii, cell types, bins and offsets into slot order in one
    // pass (slot s is sorted position s, so the sort's bins are the slots')
    CK(cudaMemcpyAsync(S.colstart[0], S.colstart[1], sizeof(int) * (ncols + 1), cudaMemcpyDeviceToDevice, st));
    LAUNCH(launch_load_slots(S, src_x, src_y, src_z, src_r, src_ct, S.col[1], S.iz[1], ctx->uperm, grd, blk, st));
    // the other fields
    auto up_d = [&](const double *src, double *dst, double fill) -> int {
        if (src) {
            CK(cudaMemcpyAsync(ctx->ud, src, sizeof(double) * n, kind, st));
            LAUNCH(launch_gather_d(dst, ctx->ud, ctx->uperm, (int)n, grd, blk, st));
        } else if (fill == 0.0) {
            CK(cudaMemsetAsync(dst, 0, sizeof(double) * n, st));
        } else {
            std::vector<double> h((size_t)n, fill);
            CK(cudaMemcpyAsync(ctx->ud, h.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
            CK(cudaStreamSynchronize(st));
            CK(cudaMemcpyAsync(dst, ctx->ud, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        }
        return BMXG_OK;
    };
    auto up_i = [&](const int32_t *src, int *dst, int planes, int fill) -> int {
        if (src) {
            CK(cudaMemcpyAsync(ctx->ui, src, sizeof(int) * n * planes, kind, st));
            LAUNCH(launch_gather_i(dst, ctx->ui, ctx->uperm, (int)n, planes, grd, blk, st));
        } else {
            CK(cudaMemsetAsync(dst, fill == 0 ? 0 : 0xff, sizeof(int) * n * planes, st));
        }
        return BMXG_OK;
    };
    if ((rc = up_d(p->velx, S.vx, 0.0))) return rc;
    if ((rc = up_d(p->vely, S.vy, 0.0))) return rc;
    if ((rc = up_d(p->velz, S.vz, 0.0))) return rc;
    if ((rc = up_d(p->wx, S.wx, 0.0))) return rc;
    if ((rc = up_d(p->wy, S.wy, 0.0))) return rc;
    if ((rc = up_d(p->wz, S.wz, 0.0))) return rc;
    if (rods) {
        if ((rc = up_d(p->c_length, S.clen, 0.0))) return rc;
        if ((rc = up_d(p->area, S.area, 0.0))) return rc;
        if ((rc = up_d(p->bond_scale, S.bscale, 1.0))) return rc;
        if ((rc = up_d(p->theta, S.theta[0], 0.0))) return rc;
        if ((rc = up_d(p->phi, S.phi[0], 0.0))) return rc;
        if ((rc = up_i(p->id, S.id, 1, 0))) return rc;
        if ((rc = up_i(p->cpu, S.cpu, 1, 0))) return rc;
        if ((rc = up_i(p->fuse_tip, S.fuse_tip, 1, 0))) return rc;
        if ((rc = up_i(p->position, S.position, 1, 0))) return rc;
        if ((rc = up_i(p->fix_site, S.fix_site, 1, 0))) return rc;
        if ((rc = up_i(p->fuse_flag, S.fflag, 1, 0))) return rc;
        if ((rc = up_i(p->split_flag, S.sflag, 1, 0))) return rc;
        if ((rc = up_i(p->new_flag, S.nflag, 1, 0))) return rc;
        if ((rc = up_i(p->dltd, S.dltd, 6, -1))) return rc;
        // bond table planes: n_bnds, ids[4], cpus[4], sites[4]
        if ((rc = up_i(p->n_bnds, S.tab[0], 1, 0))) return rc;
        if ((rc = up_i(p->seg_id1, S.tab[0] + n, 4, 0))) return rc;
        if ((rc = up_i(p->seg_id2, S.tab[0] + 5 * n, 4, 0))) return rc;
        if ((rc = up_i(p->site, S.tab[0] + 9 * n, 4, 0))) return rc;
        LAUNCH(launch_trig(S, 0, grd, blk, st));
        LAUNCH(launch_rod_mobility(S, dev_params(ctx->prm), grd, blk, st));
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(ctx->h_cnt, ctx->d_cnt, sizeof(DevCounters), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (ctx->h_cnt->bad_index) return fail(ctx, BMXG_ERR_STATE, "internal: inconsistent bin counts in the load sort");
    ctx->have_state = true;
    ctx->stepped = false;
    ctx->vel32 = false;
    ctx->vel64_zero = !p->velx && !p->vely && !p->velz && !p->wx && !p->wy && !p->wz;
    ctx->step_count = 0;
    ctx->parity = 0;
    ctx->rmax = rmax;
    ctx->list_valid = false;
    ctx->pcap_valid = false;
    ctx->fx_ahead = false;
    ctx->bins_exact = true;
    ctx->d_adh = nullptr;  // per-particle adhesion must be given again for the new state
    free_adjoint(ctx);
    std::memset(&ctx->stats, 0, sizeof(ctx->stats));
    ctx->stats.n_particles = n;
    return BMXG_OK;
}

int bmxg_get_state(bmxg_ctx *ctx, bmxg_particles *p, int where)
{
    if (!ctx) return BMXG_ERR_ARG;
    (void)cudaGetLastError();  // drop a non-sticky error another library left on this thread
    if (!ctx->have_state) return fail(ctx, BMXG_ERR_STATE, "no state loaded");
    if (!p || p->n != ctx->n) return fail(ctx, BMXG_ERR_ARG, "particle count differs from the loaded state");
    if (where != BMXG_HOST && where != BMXG_DEVICE) return fail(ctx, BMXG_ERR_ARG, "bad `where`");
    // positions still in the list's fixed point: host arrays asking for x, y
    // and z get each axis converted as it is stored (one pass instead of a
    // conversion and a scatter); otherwise all three are converted first
    const bool fx_store = ctx->fx_ahead && where == BMXG_HOST && p->x && p->y && p->z;
    if (!fx_store) {
        if (int rc = sync_fp64(ctx)) return rc;
    }
    const int64_t n = ctx->n;
    if (n == 0) return BMXG_OK;
    const DevState &S = ctx->S;
    cudaStream_t st = ctx->stream, st1 = ctx->io_stream;
    const bool host = where == BMXG_HOST;
    const int blk = ctx->sh_misc.block;
    const int grd = grid_for(ctx, ctx->sh_misc, n);
    const int a = ctx->parity;
    // Device arrays receive the caller-order scatter directly.  Host arrays:
    // each field is scattered into one of two staging halves on the compute
    // stream and copied out on the copy stream, so that the copy of one field
    // overlaps the scatter of the next.
    JoinIo join{nullptr};
    int used = 0;
    const bool pipe = host;  // (copies on `st` instead measured slower at every size)
    if (host) {
        int rc0 = ensure_io(ctx, (size_t)n * 48 + 256);
        if (rc0) return rc0;
    }
    if (pipe) {
        CK(cudaEventRecord(ctx->io_ev[0], st));
        CK(cudaStreamWaitEvent(st1, ctx->io_ev[0], 0));
        join.s = st1;
    }
    char *half[2] = {ctx->io_buf, ctx->io_buf + (size_t)n * 24 + 128};
    // destination of the next field: the caller's array or a staging half
    cudaError_t wait_err = cudaSuccess;
    auto begin = [&](void *dst) -> void * {
        if (!host) return dst;
        const int h = used & 1;
        if (pipe && used >= 2) {  // the half's previous copy-out is done
            const cudaError_t e = cudaStreamWaitEvent(st, ctx->io_ev[4 + h], 0);
            if (e != cudaSuccess) wait_err = e;
        }
        return half[h];
    };
    auto finish = [&](void *dst, size_t bytes) -> int {
        if (!host) return BMXG_OK;
        CK(wait_err);
        const int h = used & 1;
        CK(cudaEventRecord(ctx->io_ev[2 + h], st));
        CK(cudaStreamWaitEvent(st1, ctx->io_ev[2 + h], 0));
        CK(cudaMemcpyAsync(dst, half[h], bytes, cudaMemcpyDeviceToHost, st1));
        CK(cudaEventRecord(ctx->io_ev[4 + h], st1));
        ++used;
        return BMXG_OK;
    };
    auto out_d = [&](double *dst, const double *src) -> int {
        if (!dst || !src) return BMXG_OK;
        double *o = (double *)begin(dst);
        LAUNCH(launch_scatter_d(o, src, S.orig, (int)n, grd, blk, st));
        return finish(dst, sizeof(double) * n);
    };
    auto out_i = [&](int32_t *dst, const int *src, int planes) -> int {
        if (!dst || !src) return BMXG_OK;
        int *o = (int *)begin(dst);
        LAUNCH(launch_scatter_i(o, src, S.orig, (int)n, planes, grd, blk, st));
        return finish(dst, sizeof(int) * n * planes);
    };
    auto out_f = [&](double *dst, const float *src) -> int {  // FP32F velocities, widened
        if (!dst || !src) return BMXG_OK;
        double *o = (double *)begin(dst);
        LAUNCH(launch_scatter_f2d(o, src, S.orig, (int)n, grd, blk, st));
        return finish(dst, sizeof(double) * n);
    };
    int rc;
    if (fx_store) {
        double *dst[3] = {p->x, p->y, p->z};
        for (int ax = 0; ax < 3; ++ax) {
            double *o = (double *)begin(dst[ax]);
            LAUNCH(launch_list_to_fp64_axis(S, a, ax, o, blk, st));
            if ((rc = finish(dst[ax], sizeof(double) * n))) return rc;
        }
        ctx->fx_ahead = false;
    } else {
        if ((rc = out_d(p->x, S.x[a]))) return rc;
        if ((rc = out_d(p->y, S.y[a]))) return rc;
        if ((rc = out_d(p->z, S.z[a]))) return rc;
    }
    if (ctx->vel32) {
        if ((rc = out_f(p->velx, S.vxf))) return rc;
        if ((rc = out_f(p->vely, S.vyf))) return rc;
        if ((rc = out_f(p->velz, S.vzf))) return rc;
    } else {
        if ((rc = out_d(p->velx, S.vx))) return rc;
        if ((rc = out_d(p->vely, S.vy))) return rc;
        if ((rc = out_d(p->velz, S.vz))) return rc;
    }
    if ((rc = out_d(p->wx, S.wx))) return rc;
    if ((rc = out_d(p->wy, S.wy))) return rc;
    if ((rc = out_d(p->wz, S.wz))) return rc;
    if (S.has_rods) {
        if ((rc = out_d(p->theta, S.theta[a]))) return rc;
        if ((rc = out_d(p->phi, S.phi[a]))) return rc;
        if ((rc = out_i(p->n_bnds, S.tab[a], 1))) return rc;
        if ((rc = out_i(p->seg_id1, S.tab[a] + n, 4))) return rc;
        if ((rc = out_i(p->seg_id2, S.tab[a] + 5 * n, 4))) return rc;
        if ((rc = out_i(p->site, S.tab[a] + 9 * n, 4))) return rc;
        if ((rc = out_i(p->position, S.position, 1))) return rc;
        if ((rc = out_i(p->fix_site, S.fix_site, 1))) return rc;
        if ((rc = out_i(p->fuse_flag, S.fflag, 1))) return rc;
        if ((rc = out_i(p->split_flag, S.sflag, 1))) return rc;
        if ((rc = out_i(p->new_flag, S.nflag, 1))) return rc;
        if ((rc = out_i(p->dltd, S.dltd, 6))) return rc;
    } else if (ctx->stepped && where == BMXG_HOST) {
        // spheres: the step only clears the fusion flags (bmx_pc_interaction.cpp:178-180)
        for (int32_t *f : {p->fuse_flag, p->split_flag, p->new_flag})
            if (f) std::memset(f, 0, sizeof(int32_t) * n);
    } else if (ctx->stepped) {
        for (int32_t *f : {p->fuse_flag, p->split_flag, p->new_flag})
            if (f) CK(cudaMemsetAsync(f, 0, sizeof(int32_t) * n, st));
    }
    CK(cudaStreamSynchronize(st));
    if (pipe) CK(cudaStreamSynchronize(st1));
    return BMXG_OK;
}

}  // extern "C"

namespace {

// Enqueue one DEM step reading buffer a.  resync: the FP32F sphere step
// re-derives every slot's offsets and bin from its FP64 position.
// profiling mode: an event pair around the force kernel of this step
void prof_events(bmxg_ctx *ctx, cudaEvent_t *k0, cudaEvent_t *k1)
{
    *k0 = *k1 = nullptr;
    if (!ctx->profiling) return;
    while (ctx->kev.size() < 2 * (ctx->kev_used + 1)) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) break;
        ctx->kev.push_back(e);
    }
    if (ctx->kev.size() >= 2 * (ctx->kev_used + 1)) {
        *k0 = ctx->kev[2 * ctx->kev_used];
        *k1 = ctx->kev[2 * ctx->kev_used + 1];
        ++ctx->kev_used;
    }
}

// ---- FP32F neighbour list with a skin ---------------------------------------
constexpr int kListMaxAge = 64;      // builds at least this often
constexpr int kListMinSteps = 2;     // a shorter first call after a load runs the per-step path

// Skin of the list for the loaded state and parameters, or 0 where the list
// would not reproduce the reference's pair set: the largest cutoff
// 2 r_max + bw plus the skin must stay within the smallest bin width (so
// that every pair inside the cutoff is a stencil pair whatever the bins),
// BMXCheckPair must hold for every stencil pair, and the fixed point's high
// word must resolve offsets to 2^-20 of a bin.
float list_skin(const bmxg_ctx *ctx)
{
    if (ctx->S.has_rods || ctx->n == 0 || ctx->n >= (1LL << kNbrShift)) return 0.0f;
    if (ctx->ncells_total >= (1LL << 30)) return 0.0f;  // 3D cell offsets of the build
    double skin = 1e300;
    for (const DevGeom &g : ctx->h_geoms) {
        if (!g.nbh_trivial) return 0.0f;
        const double dmin = std::min(g.dx[0], std::min(g.dx[1], g.dx[2]));
        const double rcut = 2.0 * ctx->rmax + ctx->prm.bndry_width;
        const double sk = std::min(0.25 * dmin, 0.95 * (dmin - rcut));
        if (!(sk >= 0.02 * dmin)) return 0.0f;
        for (int d = 0; d < 3; ++d)
            if (!(std::ldexp((g.per[d] ? 1.0 : 4.0) * g.len[d], -32) <= std::ldexp(dmin, -20))) return 0.0f;
        skin = std::min(skin, sk);
    }
    return (float)skin;
}

// Allocate the list on first use; (re)initialise its control block when the
// state or the skin changed, asking the next step for a build.
int ensure_list(bmxg_ctx *ctx, float skin)
{
    DevState &S = ctx->S;
    if (!S.nbr) {
        int rc;
        if ((rc = dalloc(ctx, &S.nbr, (size_t)(kNbrCap - kNbrInline) * ctx->n))) return rc;
        if ((rc = dalloc(ctx, &S.lrec, ctx->n))) return rc;
        const size_t ngroups = ((size_t)ctx->n + 31) / 32;
        if ((rc = dalloc(ctx, &S.xcnt, ngroups))) return rc;
        if ((rc = dalloc(ctx, &S.xoff, ngroups + 1))) return rc;
        if ((rc = dalloc(ctx, &S.xlist, (size_t)(kNbrCap - kNbrInline) * ctx->n))) return rc;
        for (int k = 0; k < 2; ++k) {
            if ((rc = dalloc(ctx, &S.fxh[k], ctx->n))) return rc;
            if ((rc = dalloc(ctx, &S.fxl[k], 3 * (size_t)ctx->n))) return rc;
        }
        if ((rc = dalloc(ctx, &S.cellstart, ctx->ncells_total + 1))) return rc;
        // (the scratch serves the scan of the column counts and that of the groups' entries)
        const int nscan = (int)std::max<int64_t>(S.ncols_total, ((int64_t)ctx->n + 31) / 32);
        if ((rc = dalloc(ctx, &ctx->cell_scratch, scan_scratch_ints(nscan)))) return rc;
        if ((rc = dalloc(ctx, &S.lctl, 1))) return rc;
        S.ncells_total = (int)ctx->ncells_total;
        S.cols_max = 0;
        for (const DevGeom &g : ctx->h_geoms) S.cols_max = std::max(S.cols_max, g.n[0] * g.n[1]);
        // offsets within [0, n] from the start, whatever a build leaves unwritten
        CK(cudaMemsetAsync(S.cellstart, 0, sizeof(int) * (ctx->ncells_total + 1), ctx->stream));
        ctx->list_valid = false;
        drop_graphs(ctx);  // captured kernels hold the state's pointers by value
    }
    if (ctx->list_valid && skin == ctx->skin_cur) return BMXG_OK;
    double dmax = 0.0;
    for (const DevGeom &g : ctx->h_geoms) dmax = std::max(dmax, std::max(g.dx[0], std::max(g.dx[1], g.dx[2])));
    ListCtl h;
    std::memset(&h, 0, sizeof(h));
    h.skin = skin;
    h.eps_step = (float)(4.0e-7 * dmax);
    for (int k = 0; k < 3; ++k) {  // empty spreads (see k_list_decide)
        h.inc_min[k] = 0xff800000u;
        h.inc_max[k] = 0x007fffffu;
    }
    h.max_age = kListMaxAge;
    h.force = 1;
    // the fixed-point positions start from the FP64 ones
    LAUNCH(launch_list_init(S, ctx->parity, grid_for(ctx, ctx->sh_misc, ctx->n), ctx->sh_misc.block, ctx->stream));
    ctx->fx_ahead = false;
    CK(cudaMemcpyAsync(S.lctl, &h, sizeof(h), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->skin_cur = skin;
    ctx->body_runs_seen = 0;
    ctx->list_valid = true;
    return BMXG_OK;
}

// Bins of buffer `parity` as the reference has them (after list steps froze
// them); every consumer of the bins other than a list step calls this.
// FP64 positions of buffer `parity` from the list path's fixed point, when
// list steps ran since they were last written; every reader of the FP64
// positions calls this first.
int sync_fp64(bmxg_ctx *ctx)
{
    if (!ctx->fx_ahead || !ctx->have_state || ctx->n == 0) return BMXG_OK;
    LAUNCH(launch_list_to_fp64(ctx->S, ctx->parity, grid_for(ctx, ctx->sh_misc, ctx->n), ctx->sh_misc.block,
                               ctx->stream));
    ctx->fx_ahead = false;
    return BMXG_OK;
}

int ensure_exact(bmxg_ctx *ctx)
{
    if (int rc = sync_fp64(ctx)) return rc;
    if (ctx->bins_exact || !ctx->have_state) return BMXG_OK;
    const int blk = ctx->sh_misc.block, grd = grid_for(ctx, ctx->sh_misc, ctx->n);
    LAUNCH(launch_bin(ctx->S, ctx->parity, grd, blk, ctx->stream));
    LAUNCH(launch_rebuild(ctx->S, ctx->parity, ctx->scan_scratch, grd, blk, ctx->stream));
    ctx->bins_exact = true;
    ctx->list_valid = false;
    return BMXG_OK;
}

// One FP32F list step: decide, build when needed (a conditional node when
// capturing), then the force / update kernel.  Build kernels are counted as
// launches only when they run (ListCtl::body_runs).
int enqueue_list_step(bmxg_ctx *ctx, double dt, int a)
{
    const DevState &S = ctx->S;
    cudaStream_t st = ctx->stream;
    const DevParams P = dev_params(ctx->prm);
    // the decision kernel clears the per-step counters
    const int64_t n = ctx->n;
    const int mblk = ctx->sh_misc.block, mgrd = grid_for(ctx, ctx->sh_misc, n);
    if (ctx->capturing) {
        cudaStreamCaptureStatus cs;
        cudaGraph_t cg = nullptr;
        const cudaGraphNode_t *deps = nullptr;
        const cudaGraphEdgeData *ed = nullptr;
        size_t nd = 0;
        CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, &deps, &ed, &nd));
        cudaGraphConditionalHandle h;
        CK(cudaGraphConditionalHandleCreate(&h, cg, 0, 0));
        LAUNCH(launch_list_decide(S, (unsigned long long)h, 1, st));
        CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, &deps, &ed, &nd));
        cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeIf;
        cp.conditional.size = 1;
        cudaGraphNode_t cn = nullptr;
        CK(cudaGraphAddNode(&cn, cg, deps, ed, nd, &cp));
        CK(cudaStreamUpdateCaptureDependencies(st, &cn, nullptr, 1, cudaStreamSetCaptureDependencies));
        CK(cudaStreamBeginCaptureToGraph(ctx->body_stream, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                         cudaStreamCaptureModeRelaxed));
        launch_list_rebuild(S, P, a, ctx->cell_scratch, mgrd, mblk, ctx->lb_block, ctx->body_stream);
        const cudaError_t e1 = cudaPeekAtLastError();
        cudaGraph_t body = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(ctx->body_stream, &body);
        if (e1 != cudaSuccess || e2 != cudaSuccess)
            return fail(ctx, BMXG_ERR_CUDA,
                        std::string("list build capture: ") + cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
    } else {
        LAUNCH(launch_list_decide(S, 0, 0, st));
        launch_list_rebuild(S, P, a, ctx->cell_scratch, mgrd, mblk, ctx->lb_block, st);
        const cudaError_t e = cudaPeekAtLastError();
        if (e != cudaSuccess) return fail(ctx, BMXG_ERR_CUDA, std::string("list build: ") + cudaGetErrorString(e));
    }
    cudaEvent_t k0, k1;
    prof_events(ctx, &k0, &k1);
    if (k0) cudaEventRecord(k0, st);
    LAUNCH(launch_list_step(S, P, dt, a, ctx->nsm, ctx->ls_block, ctx->ls_passes, st, ctx->ls_persist));
    if (k1) cudaEventRecord(k1, st);
    return BMXG_OK;
}

int enqueue_step(bmxg_ctx *ctx, double dt, int precision, int a, int resync)
{
    if (ctx->list_on) return enqueue_list_step(ctx, dt, a);
    const DevState &S = ctx->S;
    cudaStream_t st = ctx->stream;
    const DevParams P = dev_params(ctx->prm);
    const int b = a ^ 1;
    // per-step counters (out-of-domain, images, pairs, repairs); `nonfinite` is sticky
    cudaMemsetAsync(ctx->d_cnt, 0, offsetof(DevCounters, nonfinite), st);
    cudaMemsetAsync(&ctx->d_cnt->pairs, 0, sizeof(DevCounters) - offsetof(DevCounters, pairs), st);
    const int64_t n = ctx->n;
    const int mblk = ctx->sh_misc.block, mgrd = grid_for(ctx, ctx->sh_misc, n);
    cudaEvent_t k0, k1;
    prof_events(ctx, &k0, &k1);
    if (!S.has_rods) {
        const Shape &sh = ctx->sh_sphere[precision == BMXG_FP32F ? 1 : 0];
        if (k0) cudaEventRecord(k0, st);
        int sg, sb;
        stencil_shape(ctx, sh, n, &sg, &sb);
        LAUNCH(launch_sphere_step(S, P, dt, a, precision, sg, sb, st, resync));
        if (k1) cudaEventRecord(k1, st);
    } else {
        const int rg = grid_for(ctx, ctx->sh_rod, n);
        // FP32F: the flat pipeline over the pairs the bookkeeping records
        const bool pipe = precision == BMXG_FP32F && S.rnb;
        if (pipe) cudaMemsetAsync(S.rctl, 0, sizeof(RodCtl), st);
        LAUNCH(launch_rod_book(S, P, a, pipe, rg, ctx->sh_rod.block, st));
        if (k0) cudaEventRecord(k0, st);
        if (pipe)
            LAUNCH(launch_rod_pairs(S, P, a, ctx->nsm, (int)n, st));
        else
            LAUNCH(launch_rod_force(S, P, a, precision, rg, ctx->sh_rod.block, st));
        if (k1) cudaEventRecord(k1, st);
        LAUNCH(launch_rod_update(S, dt, a, mgrd, mblk, st));
    }
    LAUNCH(launch_rebuild(S, b, ctx->scan_scratch, mgrd, mblk, st));
    return BMXG_OK;
}

int get_graph(bmxg_ctx *ctx, double dt, int precision, int parity, cudaGraphExec_t *out, int single = -1)
{
    GraphKey key{dt, precision, parity, single};
    auto it = ctx->graphs.find(key);
    if (it != ctx->graphs.end()) {
        *out = it->second;
        return BMXG_OK;
    }
    // kResyncEvery steps (an even number, so the graph ends on the parity it
    // starts from); the FP32F re-sync falls on its last step
    cudaGraph_t g = nullptr;
    const int64_t before = ctx->launches;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int rc2 = BMXG_OK;
    ctx->capturing = true;
    if (single >= 0)
        rc2 = enqueue_step(ctx, dt, precision, parity, single);
    else
        for (int s = 0; s < kResyncEvery && !rc2; ++s)
            rc2 = enqueue_step(ctx, dt, precision, parity ^ (s & 1), s == kResyncEvery - 1);
    ctx->capturing = false;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (rc2) {
        if (g) cudaGraphDestroy(g);
        ctx->launches = before;
        return rc2;
    }
    ctx->graph_kernels[key] = (int)(ctx->launches - before);  // counted per replay instead
    ctx->launches = before;
    if (e != cudaSuccess) return fail(ctx, BMXG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    cudaGraphExec_t ex = nullptr;
    e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(ctx, BMXG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    ctx->graphs[key] = ex;
    *out = ex;
    return BMXG_OK;
}

// What a call of nsteps steps in this form needs before it enqueues them:
// the list or exact bins, the buffers of the path it takes (graphs captured
// before an allocation are dropped: they hold the state's pointers by value).
int step_setup(bmxg_ctx *ctx, int32_t nsteps, int32_t precision)
{
    float skin = (precision == BMXG_FP32F && ctx->list_mode) ? list_skin(ctx) : 0.0f;
    if (skin > 0.0f && !ctx->list_valid && nsteps < kListMinSteps && ctx->step_count == 0) skin = 0.0f;
    if (skin > 0.0f) {
        int rc = ensure_list(ctx, skin);
        if (rc) return rc;
    } else {
        int rc = ensure_exact(ctx);
        if (rc) return rc;
    }
    if ((skin > 0.0f) != ctx->list_on) drop_graphs(ctx);
    ctx->list_on = skin > 0.0f;
    ctx->pcap_valid = false;
    if (ctx->list_on && ctx->pair_capture && !ctx->S.pcap) {
        int rc = dalloc(ctx, &ctx->S.pcap, (size_t)(kPairCap + 1) * ctx->n);
        if (rc) return rc;
        drop_graphs(ctx);
    }
    if (ctx->S.has_rods && precision == BMXG_FP32F && !ctx->S.rnb) {  // the FP32F rod pipeline's buffers
        const size_t n = (size_t)ctx->n;
        int2 *nb = nullptr, *work = nullptr;
        int *cnt = nullptr;
        double *res = nullptr;
        RodCtl *ctl = nullptr;
        int rc = dalloc(ctx, &nb, n * kRodCap);
        if (!rc) rc = dalloc(ctx, &cnt, n);
        if (!rc) rc = dalloc(ctx, &res, n * kRodCap * 6);
        if (!rc) rc = dalloc(ctx, &work, n * kRodCap);
        if (!rc) rc = dalloc(ctx, &ctl, 1);
        if (rc) return rc;
        ctx->S.rnb = nb;
        ctx->S.rcnt = cnt;
        ctx->S.rres = res;
        ctx->S.rwork = work;
        ctx->S.rctl = ctl;
        drop_graphs(ctx);
    }
    return BMXG_OK;
}

}  // namespace

extern "C" {

int bmxg_prepare(bmxg_ctx *ctx, double dt, int32_t precision)
{
    if (!ctx) return BMXG_ERR_ARG;
    ctx->vel64_zero = false;  // (its kernels may write the FP64 velocity planes)
    (void)cudaGetLastError();  // drop a non-sticky error another library left on this thread
    if (!ctx->have_state) return fail(ctx, BMXG_ERR_STATE, "no state loaded");
    if (!std::isfinite(dt)) return fail(ctx, BMXG_ERR_ARG, "bad dt");
    if (precision != BMXG_FP64 && precision != BMXG_FP32F) return fail(ctx, BMXG_ERR_ARG, "bad precision");
    if (ctx->n == 0 || ctx->profiling) return BMXG_OK;
    const double subdt = dt / 1.0;
    if (int rc = step_setup(ctx, 2 * kResyncEvery, precision)) return rc;
    // the replayed graph of kResyncEvery steps and the one-step graphs (with and
    // without the re-sync), from either parity
    for (int parity = 0; parity < 2; ++parity) {
        cudaGraphExec_t g = nullptr;
        if (int rc = get_graph(ctx, subdt, precision, parity, &g)) return rc;
        for (int resync = 0; resync < 2; ++resync)
            if (int rc = get_graph(ctx, subdt, precision, parity, &g, resync)) return rc;
    }
    return BMXG_OK;
}

int bmxg_step(bmxg_ctx *ctx, double dt, int32_t nsteps, int32_t precision)
{
    if (!ctx) return BMXG_ERR_ARG;
    // an FP32F sphere step writes the FP32 velocity planes only
    if (precision != BMXG_FP32F || ctx->S.has_rods) ctx->vel64_zero = false;
    (void)cudaGetLastError();  // drop a non-sticky error another library left on this thread
    if (!ctx->have_state) return fail(ctx, BMXG_ERR_STATE, "no state loaded");
    if (nsteps < 0 || !std::isfinite(dt)) return fail(ctx, BMXG_ERR_ARG, "bad dt or nsteps");
    if (precision != BMXG_FP64 && precision != BMXG_FP32F) return fail(ctx, BMXG_ERR_ARG, "bad precision");
    if (ctx->n == 0 || nsteps == 0) return BMXG_OK;
    // nsubsteps = ceil(dt / dtsolid) with dtsolid := dt, subdt = dt / nsubsteps
    // (bmx_pc_interaction.cpp:56-65): one substep of dt / 1
    const double subdt = dt / 1.0;
    // FP32F spheres use the neighbour list wherever it reproduces the pair set,
    // and where the steps are many enough to amortise a build: the first call
    // after a load, if shorter than kListMinSteps, takes the per-step path (a
    // load-step-store caller never reuses a list); later calls build one
    if (int rc = step_setup(ctx, nsteps, precision)) return rc;
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    int32_t left = nsteps;
    ctx->kev_used = 0;
    auto eager = [&]() -> int {  // one step on the re-sync schedule
        // re-sync on the last step of each kResyncEvery (not right after a load,
        // whose offsets are exact)
        const int resync = (ctx->step_count % kResyncEvery == kResyncEvery - 1) ? 1 : 0;
        if (ctx->profiling) {  // launched one by one, with events around the force kernel
            int rc = enqueue_step(ctx, subdt, precision, ctx->parity, resync);
            if (rc) return rc;
        } else {  // a captured one-step graph: one launch instead of the step's kernels and copies
            cudaGraphExec_t g1 = nullptr;
            int rc = get_graph(ctx, subdt, precision, ctx->parity, &g1, resync);
            if (rc) return rc;
            CK(cudaGraphLaunch(g1, ctx->stream));
            ctx->launches += ctx->graph_kernels[GraphKey{subdt, precision, ctx->parity, resync}];
        }
        ctx->parity ^= 1;
        ++ctx->step_count;
        --left;
        return BMXG_OK;
    };
    // eager steps up to the next re-sync boundary, graph replays of
    // kResyncEvery steps, eager remainder; every step eager when profiling
    while (left > 0 && (ctx->profiling || ctx->step_count % kResyncEvery != 0 || left < kResyncEvery)) {
        int rc = eager();
        if (rc) return rc;
    }
    if (left >= kResyncEvery) {
        cudaGraphExec_t g = nullptr, g_other = nullptr;
        int rc = get_graph(ctx, subdt, precision, ctx->parity, &g);
        // the other parity's graph too, so that a later call needs no capture
        if (!rc) rc = get_graph(ctx, subdt, precision, ctx->parity ^ 1, &g_other);
        if (rc) return rc;
        const int per = ctx->graph_kernels[GraphKey{subdt, precision, ctx->parity, -1}];
        while (left >= kResyncEvery) {
            CK(cudaGraphLaunch(g, ctx->stream));
            ctx->launches += per;
            ctx->step_count += kResyncEvery;
            left -= kResyncEvery;
        }
    }
    while (left > 0) {
        int rc = eager();
        if (rc) return rc;
    }
    ctx->vel32 = (precision == BMXG_FP32F) && !ctx->S.has_rods;
    ctx->pcap_valid = ctx->list_on && ctx->S.pcap != nullptr;
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    CK(cudaMemcpyAsync(ctx->h_cnt, ctx->d_cnt, sizeof(DevCounters), cudaMemcpyDeviceToHost, ctx->stream));
    if (ctx->list_on)
        CK(cudaMemcpyAsync(ctx->h_lctl, ctx->S.lctl, sizeof(ListCtl), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->list_on) {
        ctx->fx_ahead = true;
        const unsigned long long runs = ctx->h_lctl->body_runs - ctx->body_runs_seen;
        ctx->body_runs_seen = ctx->h_lctl->body_runs;
        ctx->launches += (int64_t)runs * kListBodyKernels;
        ctx->stats.n_rebins += (int64_t)runs;
        ctx->bins_exact = false;
    } else {
        ctx->stats.n_rebins += nsteps;
        ctx->list_valid = false;
    }
    ctx->stepped = true;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->stats.last_step_ms = ms;
    for (size_t k = 0; k < ctx->kev_used; ++k) {
        float km = 0.0f;
        if (cudaEventElapsedTime(&km, ctx->kev[2 * k], ctx->kev[2 * k + 1]) == cudaSuccess) {
            ctx->stats.main_kernel_ms += km;
            ctx->stats.main_kernel_launches += 1;
        }
    }
    ctx->kev_used = 0;
    ctx->stats.n_kernel_launches = ctx->launches;
    ctx->stats.n_out_of_domain = (int64_t)ctx->h_cnt->out_of_domain;
    ctx->stats.n_edge_ghost = (int64_t)ctx->h_cnt->edge_ghost;
    ctx->stats.n_bond_repairs = (int64_t)ctx->h_cnt->bond_repairs;
    if (ctx->h_cnt->bad_index) return fail(ctx, BMXG_ERR_STATE, "internal: inconsistent bin counts");
    if (ctx->h_cnt->nonfinite) return fail(ctx, BMXG_ERR_NONFINITE, "a step produced a non-finite position");
    if (ctx->h_cnt->range)
        return fail(ctx, BMXG_ERR_STATE, "a z left the FP32F list path's range (three quarters of a length past the domain)");
    return BMXG_OK;
}

int bmxg_evolve_particles(bmxg_ctx *ctx, double dt, double *cost_per_colony, int32_t *nsubsteps)
{
    if (!ctx) return BMXG_ERR_ARG;
    int rc = bmxg_step(ctx, dt, 1, BMXG_FP64);
    if (rc) return rc;
    if (nsubsteps) *nsubsteps = 1;
    if (cost_per_colony)  // "NumParticles" knapsack weight (bmx_pc_interaction.cpp:470-473)
        for (int c = 0; c < ctx->ncol; ++c) cost_per_colony[c] = (double)(ctx->offsets[c + 1] - ctx->offsets[c]);
    return BMXG_OK;
}

int bmxg_get_stats(const bmxg_ctx *ctx, bmxg_stats *out)
{
    if (!ctx || !out) return BMXG_ERR_ARG;
    *out = ctx->stats;
    out->n_kernel_launches = ctx->launches;
    return BMXG_OK;
}

int bmxg_set_profiling(bmxg_ctx *ctx, int32_t on)
{
    if (!ctx) return BMXG_ERR_ARG;
    ctx->profiling = on != 0;
    if (ctx->profiling) {
        ctx->stats.main_kernel_ms = 0.0;
        ctx->stats.main_kernel_launches = 0;
    }
    return BMXG_OK;
}

int bmxg_step_tile(bmxg_ctx *ctx, const bmxg_tile *tile, const bmxg_particles *reals, const bmxg_particles *ghosts,
                   double dt, int32_t where)
{
    if (!ctx) return BMXG_ERR_ARG;
    ctx->vel64_zero = false;  // (its kernels may write the FP64 velocity planes)
    (void)cudaGetLastError();  // drop a non-sticky error another library left on this thread
    if (!tile || !reals || reals->n < 0 || (ghosts && ghosts->n < 0)) return fail(ctx, BMXG_ERR_ARG, "bad arguments");
    if (where != BMXG_HOST && where != BMXG_DEVICE) return fail(ctx, BMXG_ERR_ARG, "bad `where`");
    if (!std::isfinite(dt)) return fail(ctx, BMXG_ERR_ARG, "bad dt");
    if (ctx->ncol != 1)
        return fail(ctx, BMXG_ERR_UNSUPPORTED, "a tile step takes a context of one geometry (the level's domain)");
    const int64_t nr = reals->n, ng = ghosts ? ghosts->n : 0;
    if (nr == 0) return BMXG_OK;
    if (!reals->x || !reals->y || !reals->z || !reals->radius || !reals->cell_type || !reals->velx || !reals->vely ||
        !reals->velz)
        return fail(ctx, BMXG_ERR_ARG, "reals need x, y, z, radius, cell_type and velx, vely, velz");
    if (ng && (!ghosts->x || !ghosts->y || !ghosts->z || !ghosts->radius || !ghosts->cell_type))
        return fail(ctx, BMXG_ERR_ARG, "ghosts need x, y, z, radius and cell_type");
    if (nr + ng >= (1LL << 30)) return fail(ctx, BMXG_ERR_UNSUPPORTED, "more than 2^30 particles in a tile");
    const bmxg_geometry &g = ctx->geoms[0];
    TileGeom T;
    std::memset(&T, 0, sizeof(T));
    double diag2 = 0.0;
    int64_t ncells = 1;
    for (int d = 0; d < 3; ++d) {
        T.plo[d] = g.prob_lo[d];
        T.phi[d] = g.prob_hi[d];
        T.len[d] = g.prob_hi[d] - g.prob_lo[d];
        T.n[d] = g.n_cell[d];
        const double dx = T.len[d] / (double)T.n[d];  // the whole-domain step's bin width and inverse
        T.dxi[d] = 1.0 / dx;
        T.per[d] = g.is_periodic[d] ? 1 : 0;
        if (tile->lo[d] < 0 || tile->hi[d] < tile->lo[d] || tile->hi[d] >= T.n[d])
            return fail(ctx, BMXG_ERR_ARG, "the tile is not a box of the domain's cells");
        T.lo[d] = tile->lo[d];
        T.nt[d] = tile->hi[d] - tile->lo[d] + 1;
        ncells *= T.nt[d] + 2;
        diag2 += 4.0 * dx * dx;
    }
    if (ncells >= (1LL << 30)) return fail(ctx, BMXG_ERR_UNSUPPORTED, "a tile of more than 2^30 cells");
    T.nbh_trivial = (ctx->prm.neighborhood >= diag2 * (1.0 + 1e-9)) ? 1 : 0;
    const int64_t nt = nr + ng;
    cudaStream_t st = ctx->stream;
    // stream-ordered scratch for the call
    std::vector<void *> mem;
    auto alloc = [&](auto **p, size_t count) -> bool {
        void *q = nullptr;
        if (cudaMallocAsync(&q, std::max<size_t>(count, 1) * sizeof(**p), st) != cudaSuccess) return false;
        mem.push_back(q);
        *p = reinterpret_cast<std::remove_reference_t<decltype(*p)>>(q);
        return true;
    };
    auto release = [&]() {
        for (void *q : mem) cudaFreeAsync(q, st);
        mem.clear();
    };
    TileBufs B;
    int *scratch = nullptr;
    const bool ok = alloc(&B.x, nt) && alloc(&B.y, nt) && alloc(&B.z, nt) && alloc(&B.r, nt) && alloc(&B.ct, nt) &&
                    alloc(&B.ox, nr) && alloc(&B.oy, nr) && alloc(&B.oz, nr) && alloc(&B.vx, nr) &&
                    alloc(&B.vy, nr) && alloc(&B.vz, nr) && alloc(&B.cell, nt) && alloc(&B.cnt, ncells) &&
                    alloc(&B.start, ncells + 1) && alloc(&B.fill, ncells) && alloc(&B.perm, nt) &&
                    alloc(&B.bad, 3) && alloc(&scratch, scan_scratch_ints((int)ncells));
    if (!ok) {
        release();
        (void)cudaGetLastError();
        return fail(ctx, BMXG_ERR_OOM, "tile scratch");
    }
    const cudaMemcpyKind kin = (where == BMXG_HOST) ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    const cudaMemcpyKind kout = (where == BMXG_HOST) ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    cudaError_t e = cudaSuccess;
    auto in = [&](void *dst, const void *src, size_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, kin, st);
    };
    in(B.x, reals->x, 8 * nr);
    in(B.y, reals->y, 8 * nr);
    in(B.z, reals->z, 8 * nr);
    in(B.r, reals->radius, 8 * nr);
    in(B.ct, reals->cell_type, 4 * nr);
    if (ng) {
        in(B.x + nr, ghosts->x, 8 * ng);
        in(B.y + nr, ghosts->y, 8 * ng);
        in(B.z + nr, ghosts->z, 8 * ng);
        in(B.r + nr, ghosts->radius, 8 * ng);
        in(B.ct + nr, ghosts->cell_type, 4 * ng);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(B.cnt, 0, sizeof(int) * ncells, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.fill, 0, sizeof(int) * ncells, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.bad, 0, 3 * sizeof(unsigned long long), st);
    if (e == cudaSuccess) {
        ctx->launches += launch_tile_step(B, T, dev_params(ctx->prm), dt / 1.0, (int)nr, (int)nt, scratch, ctx->nsm, st);
        e = cudaGetLastError();
    }
    unsigned long long bad[3] = {0ull, 0ull, 0ull};
    if (e == cudaSuccess) e = cudaMemcpyAsync(bad, B.bad, sizeof(bad), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess && !bad[0] && !bad[1]) {  // (non-finite positions are written, then reported)
        auto out = [&](void *dst, const void *src) {
            if (e == cudaSuccess) e = cudaMemcpyAsync(dst, src, 8 * nr, kout, st);
        };
        out(reals->x, B.ox);
        out(reals->y, B.oy);
        out(reals->z, B.oz);
        out(reals->velx, B.vx);
        out(reals->vely, B.vy);
        out(reals->velz, B.vz);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    release();
    if (e != cudaSuccess) return fail(ctx, BMXG_ERR_CUDA, std::string("tile step: ") + cudaGetErrorString(e));
    if (bad[1]) return fail(ctx, BMXG_ERR_UNSUPPORTED, "the tile step takes spheres (YEAST) only");
    if (bad[0])
        return fail(ctx, BMXG_ERR_ARG, "a real particle outside the tile or a ghost outside its one-cell halo");
    if (bad[2]) return fail(ctx, BMXG_ERR_NONFINITE, "a tile step produced a non-finite position");
    return BMXG_OK;
}

int bmxg_set_pair_capture(bmxg_ctx *ctx, int32_t on)
{
    if (!ctx) return BMXG_ERR_ARG;
    if ((on != 0) != ctx->pair_capture) drop_graphs(ctx);  // captured steps hold S by value
    ctx->pair_capture = on != 0;
    if (!ctx->pair_capture) ctx->S.pcap = nullptr;  // the buffer stays with the state's allocations
    ctx->pcap_valid = false;
    return BMXG_OK;
}

int bmxg_get_step_pairs(bmxg_ctx *ctx, int64_t *offs, int32_t *idx, int64_t cap, int64_t *total)
{
    if (!ctx) return BMXG_ERR_ARG;
    (void)cudaGetLastError();
    if (!offs || !total) return fail(ctx, BMXG_ERR_ARG, "offs and total are required");
    if (!ctx->pcap_valid || !ctx->S.pcap) return fail(ctx, BMXG_ERR_STATE, "no list step recorded with capture on");
    const int64_t n = ctx->n;
    const size_t w = kPairCap + 1;
    std::vector<int> rec((size_t)n * w), orig((size_t)n);
    cudaStream_t st = ctx->stream;
    CK(cudaMemcpyAsync(rec.data(), ctx->S.pcap, sizeof(int) * rec.size(), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(orig.data(), ctx->S.orig, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    std::vector<int64_t> slot_of((size_t)n);
    for (int64_t i = 0; i < n; ++i) slot_of[(size_t)orig[(size_t)i]] = i;
    offs[0] = 0;
    bool over = false;
    for (int64_t o = 0; o < n; ++o) {
        const int k = rec[(size_t)slot_of[(size_t)o] * w];
        over |= k > kPairCap;
        offs[o + 1] = offs[o] + std::min(k, kPairCap);
    }
    *total = offs[n];
    if (over) return fail(ctx, BMXG_ERR_CAPACITY, "a particle had more gated pairs than the capture holds");
    if (offs[n] > cap) return fail(ctx, BMXG_ERR_CAPACITY, "pair buffer too small");
    if (!idx) return BMXG_OK;
    for (int64_t o = 0; o < n; ++o) {
        const int *r = &rec[(size_t)slot_of[(size_t)o] * w];
        for (int k = 0; k < r[0]; ++k) idx[offs[o] + k] = orig[(size_t)r[1 + k]];
    }
    return BMXG_OK;
}

int bmxg_get_pairs(bmxg_ctx *ctx, int64_t *offs, int32_t *idx, int8_t *img, int64_t cap, int64_t *total)
{
    if (!ctx) return BMXG_ERR_ARG;
    (void)cudaGetLastError();  // drop a non-sticky error another library left on this thread
    if (!ctx->have_state) return fail(ctx, BMXG_ERR_STATE, "no state loaded");
    if (!offs || !total) return fail(ctx, BMXG_ERR_ARG, "offs and total are required");
    const int64_t n = ctx->n;
    offs[0] = 0;
    *total = 0;
    if (n == 0) return BMXG_OK;
    if (int rc0 = ensure_exact(ctx)) return rc0;
    cudaStream_t st = ctx->stream;
    const DevParams P = dev_params(ctx->prm);
    int64_t *d_offs = nullptr;
    CK(cudaMallocAsync((void **)&d_offs, sizeof(int64_t) * (n + 1), st));
    const int blk = ctx->sh_misc.block, grd = grid_for(ctx, ctx->sh_misc, n);
    ctx->launches += launch_pairs(ctx->S, P, ctx->parity, d_offs, nullptr, nullptr, 0, grd, blk, st);
    std::vector<int64_t> cnt((size_t)n);
    cudaError_t e = cudaMemcpyAsync(cnt.data(), d_offs, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaFreeAsync(d_offs, st);
        return fail(ctx, BMXG_ERR_CUDA, cudaGetErrorString(e));
    }
    for (int64_t i = 0; i < n; ++i) offs[i + 1] = offs[i] + cnt[(size_t)i];
    *total = offs[n];
    ctx->stats.n_pairs_last = offs[n];
    if (offs[n] > cap || !idx || !img) {
        cudaFreeAsync(d_offs, st);
        cudaStreamSynchronize(st);
        return (offs[n] > cap) ? fail(ctx, BMXG_ERR_CAPACITY, "pair buffer too small") : BMXG_OK;
    }
    int *d_idx = nullptr;
    int8_t *d_img = nullptr;
    const int64_t m = std::max<int64_t>(offs[n], 1);
    e = cudaMallocAsync((void **)&d_idx, sizeof(int) * m, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&d_img, m, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_offs, offs, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        ctx->launches += launch_pairs(ctx->S, P, ctx->parity, d_offs, d_idx, d_img, 1, grd, blk, st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(idx, d_idx, sizeof(int) * offs[n], cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(img, d_img, offs[n], cudaMemcpyDeviceToHost, st);
    if (d_idx) cudaFreeAsync(d_idx, st);
    if (d_img) cudaFreeAsync(d_img, st);
    cudaFreeAsync(d_offs, st);
    cudaError_t e2 = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return fail(ctx, BMXG_ERR_CUDA, cudaGetErrorString(e));
    return BMXG_OK;
}

int bmxg_particle_exchange(bmxg_ctx *ctx, const double *vol, double *conc, double dt, const double *xpar,
                           int32_t where)
{
    if (!ctx) return BMXG_ERR_ARG;
    ctx->vel64_zero = false;  // (its kernels may write the FP64 velocity planes)
    (void)cudaGetLastError();  // drop a non-sticky error another library left on this thread
    if (!ctx->have_state) return fail(ctx, BMXG_ERR_STATE, "no state loaded");
    if (!vol || !conc || !xpar || !std::isfinite(dt)) return fail(ctx, BMXG_ERR_ARG, "vol, conc, xpar and a finite dt are required");
    if (where != BMXG_HOST && where != BMXG_DEVICE) return fail(ctx, BMXG_ERR_ARG, "bad `where`");
    const int64_t n = ctx->n;
    if (n == 0 || !ctx->S.has_rods) return BMXG_OK;  // only FUNGI segments exchange
    if (int rc0 = ensure_exact(ctx)) return rc0;
    cudaStream_t st = ctx->stream;
    const cudaMemcpyKind in = (where == BMXG_HOST) ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    const cudaMemcpyKind back = (where == BMXG_HOST) ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    double *buf = nullptr;  // caller-order staging (3n), slot-order vol (n), conc (3n), out (3n)
    CK(cudaMallocAsync((void **)&buf, sizeof(double) * 10 * n, st));
    double *stage = buf, *svol = buf + 3 * n, *sc = buf + 4 * n, *so = buf + 7 * n;
    const int blk = ctx->sh_misc.block, grd = grid_for(ctx, ctx->sh_misc, n);
    cudaError_t e = cudaMemcpyAsync(stage, vol, sizeof(double) * n, in, st);
    int launched = 0;
    if (e == cudaSuccess) {
        launched += launch_gather_d(svol, stage, ctx->S.orig, (int)n, grd, blk, st);
        e = cudaMemcpyAsync(stage, conc, sizeof(double) * 3 * n, in, st);
    }
    if (e == cudaSuccess) {
        for (int k = 0; k < 3; ++k)
            launched += launch_gather_d(sc + (size_t)k * n, stage + (size_t)k * n, ctx->S.orig, (int)n, grd, blk, st);
        launched += launch_exchange(ctx->S, dev_params(ctx->prm), ctx->parity, svol, sc, so, dt, xpar, grd, blk, st);
        for (int k = 0; k < 3; ++k)
            launched += launch_scatter_d(stage + (size_t)k * n, so + (size_t)k * n, ctx->S.orig, (int)n, grd, blk, st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(conc, stage, sizeof(double) * 3 * n, back, st);
    cudaFreeAsync(buf, st);
    const cudaError_t e2 = cudaStreamSynchronize(st);
    ctx->launches += launched;
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return fail(ctx, BMXG_ERR_CUDA, std::string("particle exchange: ") + cudaGetErrorString(e));
    return BMXG_OK;
}

int bmxg_set_list_mode(bmxg_ctx *ctx, int32_t mode)
{
    if (!ctx) return BMXG_ERR_ARG;
    if (mode != 0 && mode != 1) return fail(ctx, BMXG_ERR_ARG, "list mode must be 0 or 1");
    if (ctx->list_mode != mode) {
        ctx->list_mode = mode;
        ctx->list_valid = false;
        drop_graphs(ctx);
    }
    return BMXG_OK;
}

int bmxg_init_bonds(bmxg_ctx *ctx, double rlim, int64_t *added, int64_t *overflow)
{
    if (!ctx) return BMXG_ERR_ARG;
    ctx->vel64_zero = false;  // (its kernels may write the FP64 velocity planes)
    (void)cudaGetLastError();  // drop a non-sticky error another library left on this thread
    if (added) *added = 0;
    if (overflow) *overflow = 0;
    if (!ctx->have_state) return fail(ctx, BMXG_ERR_STATE, "no state loaded");
    if (!(rlim > 0.0)) rlim = 1.0e-7;
    if (ctx->n == 0 || !ctx->S.has_rods) return BMXG_OK;
    if (int rc0 = ensure_exact(ctx)) return rc0;
    cudaStream_t st = ctx->stream;
    const DevParams P = dev_params(ctx->prm);
    unsigned long long *d_cnt = nullptr;
    CK(cudaMallocAsync((void **)&d_cnt, 2 * sizeof(unsigned long long), st));
    unsigned long long h_cnt[2] = {0, 0};
    cudaError_t e = cudaMemsetAsync(d_cnt, 0, 2 * sizeof(unsigned long long), st);
    if (e == cudaSuccess) {
        const int blk = ctx->sh_misc.block, grd = grid_for(ctx, ctx->sh_misc, ctx->n);
        ctx->launches += launch_init_bonds(ctx->S, P, ctx->parity, rlim, d_cnt, grd, blk, st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_cnt, d_cnt, sizeof(h_cnt), cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d_cnt, st);
    cudaError_t e2 = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return fail(ctx, BMXG_ERR_CUDA, cudaGetErrorString(e));
    if (added) *added = (int64_t)h_cnt[0];
    if (overflow) *overflow = (int64_t)h_cnt[1];
    if (h_cnt[1]) return fail(ctx, BMXG_ERR_CAPACITY, "a segment end met more bonds than its four table slots");
    return BMXG_OK;
}

int bmxg_autotune(bmxg_ctx *ctx, const char *cache_path)
{
    if (!ctx) return BMXG_ERR_ARG;
    ctx->vel64_zero = false;  // (its kernels may write the FP64 velocity planes)
    (void)cudaGetLastError();  // drop a non-sticky error another library left on this thread
    if (!ctx->have_state) return fail(ctx, BMXG_ERR_STATE, "no state loaded");
    if (ctx->n == 0 || ctx->S.has_rods) return BMXG_OK;
    if (int rc0 = ensure_exact(ctx)) return rc0;
    ctx->list_valid = false;  // the sweep writes the other buffer
    const int64_t n = ctx->n;
    char devname[256] = {0};
    {
        cudaDeviceProp prop;
        CK(cudaGetDeviceProperties(&prop, ctx->device));
        std::snprintf(devname, sizeof(devname), "%s", prop.name);
    }
    // the colony-size histogram (count per power-of-two size class) keys the
    // cache with the device and the particle count
    std::string hist;
    {
        int cls[64] = {0};
        for (int c = 0; c < ctx->ncol; ++c) {
            const int64_t m = ctx->offsets[c + 1] - ctx->offsets[c];
            int k = 0;
            while (k < 62 && (1LL << k) <= m) ++k;
            ++cls[k];
        }
        for (int k = 0; k < 64; ++k)
            if (cls[k]) hist += std::to_string(k) + ":" + std::to_string(cls[k]) + ",";
    }
    auto cache_read = [&]() {
        std::string txt;
        if (!cache_path) return txt;
        FILE *f = std::fopen(cache_path, "r");
        if (!f) return txt;
        char buf[4096];
        size_t r;
        while ((r = std::fread(buf, 1, sizeof(buf), f)) > 0) txt.append(buf, r);
        std::fclose(f);
        return txt;
    };
    auto cache_add = [&](const char *entry) {
        if (!cache_path) return;
        std::string txt = cache_read();
        const size_t close = txt.rfind('}');
        if (close == std::string::npos || txt.find('"') == std::string::npos)
            txt = std::string("{\n  ") + entry + "\n}\n";
        else
            txt = txt.substr(0, close) + ",\n  " + entry + "\n}\n";
        FILE *f = std::fopen(cache_path, "w");
        if (f) {
            std::fwrite(txt.data(), 1, txt.size(), f);
            std::fclose(f);
        }
    };
    // time `reps` launches after `warm` untimed ones (ms for the reps)
    auto timeit = [&](int warm, int reps, const std::function<int()> &launch, float *ms) -> int {
        for (int w = 0; w < warm; ++w) ctx->launches += launch();
        CK(cudaEventRecord(ctx->ev0, ctx->stream));
        for (int r = 0; r < reps; ++r) ctx->launches += launch();
        CK(cudaEventRecord(ctx->ev1, ctx->stream));
        CK(cudaEventSynchronize(ctx->ev1));
        CK(cudaGetLastError());
        CK(cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1));
        return BMXG_OK;
    };
    char key[768];
    char entry[1024];
    const DevState &S = ctx->S;
    const DevParams P = dev_params(ctx->prm);
    // the per-step stencil kernels of both forms
    for (int prec = 0; prec < 2; ++prec) {
        std::snprintf(key, sizeof(key), "\"%s|sphere|%d|n=%lld|ncol=%d|h=%s\"", devname, prec, (long long)n,
                      ctx->ncol, hist.c_str());
        {
            const std::string txt = cache_read();
            const size_t pos = txt.find(key);
            int bb = 0, gg = 0;
            if (pos != std::string::npos &&
                std::sscanf(txt.c_str() + pos + std::strlen(key), ": {\"block\": %d, \"grid\": %d}", &bb, &gg) == 2 &&
                bb > 0) {
                ctx->sh_sphere[prec].block = bb;
                ctx->sh_sphere[prec].grid = gg;
                continue;
            }
        }
        // sweep: the kernel reads buffer a and writes buffer b, so repeated
        // launches leave the state as it was except for the column counters,
        // which are cleared afterwards
        float best = 1e30f;
        Shape bs = ctx->sh_sphere[prec];
        const int blocks[] = {64, 128, 256};  // k_sphere is compiled with __launch_bounds__(256)
        for (int blk : blocks) {
            for (int mult = 1; mult <= 64; mult *= 2) {  // up to one slot per thread
                Shape sh;
                sh.block = blk;
                sh.grid = ctx->nsm * mult * std::max(1, 1024 / blk);
                const int grd = grid_for(ctx, sh, n);
                float ms = 0.0f;
                if (int rc = timeit(2, 5, [&]() { return launch_sphere_step(S, P, 0.0, ctx->parity, prec, grd, blk,
                                                                            ctx->stream, 0); }, &ms))
                    return rc;
                if (ms < best) {
                    best = ms;
                    bs = sh;
                }
            }
        }
        CK(cudaMemsetAsync(ctx->S.colcnt, 0, sizeof(int) * std::max(ctx->S.ncols_total, 1), ctx->stream));
        CK(cudaMemsetAsync(ctx->d_cnt, 0, sizeof(DevCounters), ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        ctx->sh_sphere[prec] = bs;
        std::snprintf(entry, sizeof(entry), "%s: {\"block\": %d, \"grid\": %d, \"ms_per_5\": %.4f}", key, bs.block,
                      bs.grid, best);
        cache_add(entry);
    }
    // the FP32F list path: k_list_step's block and passes per chunk,
    // k_list_build's block
    const float skin = ctx->list_mode ? list_skin(ctx) : 0.0f;
    if (skin > 0.0f) {
        std::snprintf(key, sizeof(key), "\"%s|list|n=%lld|ncol=%d|h=%s\"", devname, (long long)n, ctx->ncol,
                      hist.c_str());
        const std::string txt = cache_read();
        const size_t pos = txt.find(key);
        int sb = 0, sp = 0, bb = 0, pe = 0;
        if (pos != std::string::npos &&
            std::sscanf(txt.c_str() + pos + std::strlen(key),
                        ": {\"step_block\": %d, \"step_passes\": %d, \"step_persistent\": %d, \"build_block\": %d",
                        &sb, &sp, &pe, &bb) == 4 &&
            sb > 0 && bb > 0) {
            ctx->ls_block = sb;
            ctx->ls_passes = sp;
            ctx->ls_persist = pe != 0;
            ctx->lb_block = bb;
        } else {
            // a list built on the loaded positions; then the step launches read
            // buffer a and write buffer b (dt = 0), and the build launches
            // rewrite the same list: the loaded state is untouched, and the
            // list path starts afresh at the next step (list_valid = false)
            if (int rc = ensure_list(ctx, skin)) return rc;
            cudaStream_t st = ctx->stream;
            const int a = ctx->parity;
            const int mblk = ctx->sh_misc.block, mgrd = grid_for(ctx, ctx->sh_misc, n);
            LAUNCH(launch_list_decide(S, 0, 0, st));
            ctx->launches += launch_list_rebuild(S, P, a, ctx->cell_scratch, mgrd, mblk, ctx->lb_block, st);
            float best = 1e30f, best_b = 1e30f;
            int best_sb = ctx->ls_block, best_sp = ctx->ls_passes, best_bb = ctx->lb_block;
            bool best_pe = ctx->ls_persist;
            for (int blk : {64, 128, 256}) {
                // one block per chunk of 1, 2 or 4 passes; or one persistent wave
                // taking chunks of 2, 4 or 8 passes from the dispenser
                for (int pe = 0; pe < 2; ++pe) {
                    for (int passes : {1, 2, 4}) {
                        const int pp = pe ? 2 * passes : passes;
                        float ms = 0.0f;
                        if (int rc = timeit(2, 5, [&]() { return launch_list_step(S, P, 0.0, a, ctx->nsm, blk, pp,
                                                                                    st, pe != 0); }, &ms))
                            return rc;
                        if (ms < best) {
                            best = ms;
                            best_sb = blk;
                            best_sp = pp;
                            best_pe = pe != 0;
                        }
                    }
                }
                float ms = 0.0f;
                if (int rc = timeit(1, 3, [&]() { return launch_list_build(S, P, blk, st); }, &ms)) return rc;
                if (ms < best_b) {
                    best_b = ms;
                    best_bb = blk;
                }
            }
            CK(cudaMemsetAsync(ctx->d_cnt, 0, sizeof(DevCounters), st));
            CK(cudaStreamSynchronize(st));
            ctx->ls_block = best_sb;
            ctx->ls_passes = best_sp;
            ctx->ls_persist = best_pe;
            ctx->lb_block = best_bb;
            ctx->list_valid = false;
            std::snprintf(entry, sizeof(entry),
                          "%s: {\"step_block\": %d, \"step_passes\": %d, \"step_persistent\": %d, \"build_block\": "
                          "%d, \"step_ms_per_5\": %.4f, \"build_ms_per_3\": %.4f}",
                          key, best_sb, best_sp, best_pe ? 1 : 0, best_bb, best, best_b);
            cache_add(entry);
        }
    }
    drop_graphs(ctx);
    return BMXG_OK;
}

int bmxg_set_shapes(bmxg_ctx *ctx, const bmxg_shapes *in)
{
    if (!ctx) return BMXG_ERR_ARG;
    if (!in) return fail(ctx, BMXG_ERR_ARG, "no shapes");
    auto block_ok = [](int b) { return b >= 32 && b <= 256 && b % 32 == 0; };
    for (int k = 0; k < 2; ++k)
        if (!block_ok(in->sphere_block[k]) || in->sphere_grid[k] < 0)
            return fail(ctx, BMXG_ERR_ARG, "sphere block: a multiple of 32 up to 256; grid >= 0");
    if (!block_ok(in->list_step_block) || !block_ok(in->list_build_block) || in->list_step_passes < 0 ||
        in->list_step_passes > 64)
        return fail(ctx, BMXG_ERR_ARG, "list blocks: a multiple of 32 up to 256; passes 0..64");
    for (int k = 0; k < 2; ++k) {
        ctx->sh_sphere[k].block = in->sphere_block[k];
        ctx->sh_sphere[k].grid = in->sphere_grid[k];
    }
    ctx->ls_block = in->list_step_block;
    ctx->ls_passes = in->list_step_passes;
    ctx->ls_persist = in->list_step_persistent != 0;
    ctx->lb_block = in->list_build_block;
    drop_graphs(ctx);
    return BMXG_OK;
}

int bmxg_get_shapes(const bmxg_ctx *ctx, bmxg_shapes *out)
{
    if (!ctx || !out) return BMXG_ERR_ARG;
    std::memset(out, 0, sizeof(*out));
    for (int k = 0; k < 2; ++k) {
        out->sphere_block[k] = ctx->sh_sphere[k].block;
        out->sphere_grid[k] = ctx->sh_sphere[k].grid;
    }
    out->list_step_block = ctx->ls_block;
    out->list_step_passes = ctx->ls_passes;
    out->list_build_block = ctx->lb_block;
    out->list_step_persistent = ctx->ls_persist ? 1 : 0;
    return BMXG_OK;
}

}  // extern "C"

// ---- differentiation form ----------------------------------------------------
extern "C" {

int bmxg_set_ext(bmxg_ctx *ctx, const bmxg_ext *ext)
{
    if (!ctx) return BMXG_ERR_ARG;
    if (!ext || !std::isfinite(ext->damping) || !std::isfinite(ext->mu) || ext->damping < 0.0 || ext->mu < 0.0)
        return fail(ctx, BMXG_ERR_ARG, "damping and mu must be finite and >= 0");
    if (!ctx->have_state) return fail(ctx, BMXG_ERR_STATE, "load the state before its extension parameters");
    (void)cudaGetLastError();
    ctx->ext_gamma = ext->damping;
    ctx->ext_mu = ext->mu;
    const int64_t n = ctx->n;
    if (ext->adhesion && n > 0) {
        if (!ctx->adh_buf) {
            int rc = dalloc(ctx, &ctx->adh_buf, n);
            if (rc) return rc;
        }
        ctx->d_adh = ctx->adh_buf;
        cudaStream_t st = ctx->stream;
        CK(cudaMemcpyAsync(ctx->ud, ext->adhesion, sizeof(double) * n, cudaMemcpyHostToDevice, st));
        LAUNCH(launch_gather_d(ctx->d_adh, ctx->ud, ctx->S.orig, (int)n, grid_for(ctx, ctx->sh_misc, n),
                               ctx->sh_misc.block, st));
        CK(cudaStreamSynchronize(st));
    } else {
        ctx->d_adh = nullptr;  // buffer (if any) stays allocated until the state is freed
    }
    ctx->traj_T = -1;
    return BMXG_OK;
}

}  // extern "C"

namespace {

template <class T>
int dalloc_adj(bmxg_ctx *ctx, T **p, size_t count)
{
    void *q = nullptr;
    if (count == 0) count = 1;
    CK(cudaMalloc(&q, count * sizeof(T)));
    ctx->dallocs.push_back(q);
    *p = (T *)q;
    return BMXG_OK;
}

DiffParams diff_params(const bmxg_ctx *ctx)
{
    return DiffParams{ctx->ext_gamma, ctx->ext_mu, ctx->d_adh};
}

// copy the positions of buffer b into 3 planes at dst (slot order)
int save_pos(bmxg_ctx *ctx, int b, double *dst)
{
    const size_t bytes = sizeof(double) * ctx->n;
    CK(cudaMemcpyAsync(dst, ctx->S.x[b], bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemcpyAsync(dst + ctx->n, ctx->S.y[b], bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemcpyAsync(dst + 2 * ctx->n, ctx->S.z[b], bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    return BMXG_OK;
}

// load 3 position planes into buffer 0 and rebuild its bins and column lists
int load_pos(bmxg_ctx *ctx, const double *src)
{
    const size_t bytes = sizeof(double) * ctx->n;
    const DevState &S = ctx->S;
    CK(cudaMemcpyAsync(S.x[0], src, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemcpyAsync(S.y[0], src + ctx->n, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemcpyAsync(S.z[0], src + 2 * ctx->n, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    const int mblk = ctx->sh_misc.block, mgrd = grid_for(ctx, ctx->sh_misc, ctx->n);
    LAUNCH(launch_bin(S, 0, mgrd, mblk, ctx->stream));
    LAUNCH(launch_rebuild(S, 0, ctx->scan_scratch, mgrd, mblk, ctx->stream));
    ctx->parity = 0;
    return BMXG_OK;
}

int dfwd_step(bmxg_ctx *ctx, double dt)
{
    const DevState &S = ctx->S;
    const int a = ctx->parity;
    const int mblk = ctx->sh_misc.block, mgrd = grid_for(ctx, ctx->sh_misc, ctx->n);
    const Shape &sh = ctx->sh_sphere[0];
    int sg, sb;
    stencil_shape(ctx, sh, ctx->n, &sg, &sb);
    LAUNCH(launch_dfwd(S, dev_params(ctx->prm), diff_params(ctx), dt, a, sg, sb,
                       ctx->stream));
    LAUNCH(launch_rebuild(S, a ^ 1, ctx->scan_scratch, mgrd, mblk, ctx->stream));
    ctx->parity = a ^ 1;
    return BMXG_OK;
}

}  // namespace

extern "C" {

int bmxg_forward(bmxg_ctx *ctx, double dt, int32_t nsteps, int32_t ckpt_every)
{
    if (!ctx) return BMXG_ERR_ARG;
    ctx->vel64_zero = false;  // (its kernels may write the FP64 velocity planes)
    if (!ctx->have_state) return fail(ctx, BMXG_ERR_STATE, "no state loaded");
    if (ctx->S.has_rods) return fail(ctx, BMXG_ERR_UNSUPPORTED, "the differentiation form covers spheres");
    if (nsteps < 0 || ckpt_every < 1 || !std::isfinite(dt)) return fail(ctx, BMXG_ERR_ARG, "bad dt, nsteps or ckpt_every");
    (void)cudaGetLastError();
    if (int rc0 = ensure_exact(ctx)) return rc0;
    ctx->list_valid = false;
    const int64_t n = ctx->n;
    free_adjoint(ctx);
    if (n == 0) {
        ctx->traj_T = nsteps;
        ctx->traj_k = ckpt_every;
        ctx->traj_dt = dt;
        return BMXG_OK;
    }
    const int nseg = (nsteps + ckpt_every - 1) / ckpt_every;
    int rc;
    if ((rc = dalloc_adj(ctx, &ctx->ckpt, (size_t)(nseg + 1) * 3 * n))) return rc;
    if ((rc = dalloc_adj(ctx, &ctx->xT, (size_t)3 * n))) return rc;
    const double subdt = dt / 1.0;
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    for (int t = 0; t < nsteps; ++t) {
        if (t % ckpt_every == 0 && (rc = save_pos(ctx, ctx->parity, ctx->ckpt + (size_t)(t / ckpt_every) * 3 * n)))
            return rc;
        if ((rc = dfwd_step(ctx, subdt))) return rc;
    }
    if ((rc = save_pos(ctx, ctx->parity, ctx->xT))) return rc;
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    CK(cudaMemcpyAsync(ctx->h_cnt, ctx->d_cnt, sizeof(DevCounters), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->stats.last_step_ms = ms;
    ctx->stepped = true;
    ctx->traj_T = nsteps;
    ctx->traj_k = ckpt_every;
    ctx->traj_dt = subdt;
    ctx->vel32 = false;
    ctx->stats.n_kernel_launches = ctx->launches;
    if (ctx->h_cnt->bad_index) return fail(ctx, BMXG_ERR_STATE, "internal: inconsistent bin counts");
    if (ctx->h_cnt->nonfinite) return fail(ctx, BMXG_ERR_NONFINITE, "a step produced a non-finite position");
    return BMXG_OK;
}

int bmxg_backward(bmxg_ctx *ctx, const double *dL_dx, double *dL_dx0, double *dL_dparams, double *dL_dadhesion)
{
    if (!ctx) return BMXG_ERR_ARG;
    ctx->vel64_zero = false;  // (its kernels may write the FP64 velocity planes)
    if (ctx->traj_T < 0) return fail(ctx, BMXG_ERR_STATE, "bmxg_forward must run first");
    if (!dL_dx) return fail(ctx, BMXG_ERR_ARG, "dL_dx is required");
    (void)cudaGetLastError();
    const int64_t n = ctx->n;
    const int T = ctx->traj_T, K = ctx->traj_k;
    if (n == 0) {
        if (dL_dparams) dL_dparams[0] = dL_dparams[1] = dL_dparams[2] = 0.0;
        return BMXG_OK;
    }
    cudaStream_t st = ctx->stream;
    const DevState &S = ctx->S;
    int rc;
    ctx->list_valid = false;  // the recomputation rewrites buffer 0
    if (!ctx->lam[0]) {
        if ((rc = dalloc_adj(ctx, &ctx->lam[0], (size_t)3 * n))) return rc;
        if ((rc = dalloc_adj(ctx, &ctx->lam[1], (size_t)3 * n))) return rc;
        if ((rc = dalloc_adj(ctx, &ctx->segbuf, (size_t)K * 3 * n))) return rc;
        if ((rc = dalloc_adj(ctx, &ctx->gacc, (size_t)3 * n))) return rc;
        if ((rc = dalloc_adj(ctx, &ctx->gadh, (size_t)n))) return rc;
        if ((rc = dalloc_adj(ctx, &ctx->gout, 4))) return rc;
    }
    const int mblk = ctx->sh_misc.block, mgrd = grid_for(ctx, ctx->sh_misc, n);
    CK(cudaEventRecord(ctx->ev0, st));
    // dL/dx_T, caller order -> slot order
    for (int c = 0; c < 3; ++c) {
        CK(cudaMemcpyAsync(ctx->ud, dL_dx + (size_t)c * n, sizeof(double) * n, cudaMemcpyHostToDevice, st));
        LAUNCH(launch_gather_d(ctx->lam[0] + (size_t)c * n, ctx->ud, S.orig, (int)n, mgrd, mblk, st));
    }
    CK(cudaMemsetAsync(ctx->gacc, 0, sizeof(double) * 3 * n, st));
    CK(cudaMemsetAsync(ctx->gadh, 0, sizeof(double) * n, st));
    int cur = 0;
    const DevParams P = dev_params(ctx->prm);
    const DiffParams D = diff_params(ctx);
    const Shape &sh = ctx->sh_sphere[0];
    int ag, ab;
    stencil_shape(ctx, sh, n, &ag, &ab);
    const int nseg = (T + K - 1) / K;
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int c0 = seg * K, c1 = std::min(c0 + K, T);
        // recompute the segment's positions from its checkpoint
        if ((rc = load_pos(ctx, ctx->ckpt + (size_t)seg * 3 * n))) return rc;
        for (int t = c0; t < c1; ++t) {
            if ((rc = save_pos(ctx, ctx->parity, ctx->segbuf + (size_t)(t - c0) * 3 * n))) return rc;
            if (t + 1 < c1 && (rc = dfwd_step(ctx, ctx->traj_dt))) return rc;
        }
        // reverse sweep through the segment
        for (int t = c1 - 1; t >= c0; --t) {
            if ((rc = load_pos(ctx, ctx->segbuf + (size_t)(t - c0) * 3 * n))) return rc;
            LAUNCH(launch_dadj(S, P, D, ctx->traj_dt, 0, ctx->lam[cur], ctx->lam[cur ^ 1], ctx->gacc, ctx->gadh,
                               ag, ab, st));
            cur ^= 1;
        }
    }
    LAUNCH(launch_dreduce(ctx->gacc, (int)n, 3, ctx->gout, st));
    CK(cudaEventRecord(ctx->ev1, st));
    if (dL_dx0) {
        for (int c = 0; c < 3; ++c) {
            LAUNCH(launch_scatter_d(ctx->ud, ctx->lam[cur] + (size_t)c * n, S.orig, (int)n, mgrd, mblk, st));
            CK(cudaMemcpyAsync(dL_dx0 + (size_t)c * n, ctx->ud, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
        }
    }
    if (dL_dadhesion) {
        LAUNCH(launch_scatter_d(ctx->ud, ctx->gadh, S.orig, (int)n, mgrd, mblk, st));
        CK(cudaMemcpyAsync(dL_dadhesion, ctx->ud, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    }
    double g[3] = {0.0, 0.0, 0.0};
    CK(cudaMemcpyAsync(g, ctx->gout, sizeof(g), cudaMemcpyDeviceToHost, st));
    // leave the state at the end of the trajectory, as bmxg_forward did
    if ((rc = load_pos(ctx, ctx->xT))) return rc;
    CK(cudaStreamSynchronize(st));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->stats.last_step_ms = ms;
    ctx->stats.n_kernel_launches = ctx->launches;
    if (dL_dparams) {
        dL_dparams[0] = g[0];
        dL_dparams[1] = g[1];
        dL_dparams[2] = ctx->ext_mu > 0.0 ? g[2] : 0.0;
    }
    return BMXG_OK;
}

}  // extern "C"
