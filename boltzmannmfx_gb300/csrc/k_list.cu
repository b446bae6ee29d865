// k_list.cu -- FP32F sphere step over a neighbour list with a skin.
//
// The force acts only on pairs closer than rA = r_i + r_j + bw
// (maxInteractionDistance and the gate r^2 <= (r_lm - 1e-15)^2,
// bmx_cell_interaction_K.H:23-40, bmx_pc_interaction.cpp:212).  When
// rA + skin is at most the smallest bin width, any pair that close sits in
// neighbouring bins, so the reference's stencil list holds it whatever the
// binning is.  The list built here holds every pair closer than rA + skin
// at build time; while no particle has moved more than skin / 2 since, it
// still holds every pair closer than rA.  The pair set of a step is
// therefore the reference's; only the FP32 rounding of the pair math (the
// precision form) differs from it.
//
// Between builds the bins stay frozen (buffer kListBins) and the FP32
// offsets advance in the frozen frame, while the FP64 positions accumulate
// and wrap periodically every step as in the reference.  A build moves
// every frame to the bin its offset has reached (every kListExactEvery-th
// build re-bins exactly from the FP64 positions instead, which also bounds
// the FP32 drift of the offsets), rebuilds the column lists and walks the
// stencil once.  The bins need not be the reference's here: with
// rA + skin within a bin width, any binning finds the same pairs.
// k_list_decide folds each step's largest
// displacement into a bound and asks for a build when the bound reaches
// skin / 2 (or after max_age steps); inside a CUDA graph the build kernels
// sit in a conditional node that the decision switches, so a step without
// a build launches two kernels.
//
// Roofline: the step kernel streams the slot state (FP64 positions in and
// out, FP32 offsets in and out, FP32 velocities out) and the list; the
// neighbour offsets it gathers are L2-resident.  HBM bound, no contraction.
#include "bmxg_stencil.cuh"

namespace bmxg {

namespace {

constexpr unsigned kSlotMask = (1u << kNbrShift) - 1u;

// bin shift code (0, 1, 2) -> -width, 0, +width
__device__ __forceinline__ float shift_of(unsigned c, float w)
{
    return (c == 1u) ? 0.0f : ((c == 0u) ? -w : w);
}

// Order-preserving integer key of a double (-0 and +0 equal): the FP64
// compares of the periodic wrap and the domain test without the FP64 pipe.
__device__ __forceinline__ long long dkey(double v)
{
    const long long b = __double_as_longlong(v);
    return (b >= 0) ? b : -(b & 0x7fffffffffffffffLL);
}

__global__ void k_list_decide(ListCtl *c, cudaGraphConditionalHandle h, int use_h)
{
    const float m2 = __uint_as_float(c->maxd2_bits);
    c->maxd2_bits = 0u;
    const float acc = c->acc + sqrtf(m2) * 1.000001f + c->eps_step;
    const int age = c->age + 1;
    const bool rb = c->force != 0 || !(2.0f * acc <= c->skin) || age > c->max_age;
    if (rb) {
        c->exact_now = (c->force != 0 || c->builds % c->exact_every == 0) ? 1 : 0;
        c->acc = 0.0f;
        c->age = 0;
        c->force = 0;
        c->builds += 1;
        c->overflow = 0ull;
    } else {
        c->acc = acc;
        c->age = age;
    }
    c->rebuild = rb ? 1 : 0;
    if (use_h) cudaGraphSetConditional(h, rb ? 1u : 0u);
}

// Move one axis of a frozen frame to the bin the offset now falls in: the
// offset leaves [0, w) by less than the skin between builds, so the bin moves
// by at most one.  Periodic axes wrap the bin index (bin n + 1 is bin 1 one
// period on, the frame the FP64 wrap of the position matches); on a closed
// axis a bin outside 1..n keeps its frame, as bin_of clamps there.
__device__ __forceinline__ void reframe(float &r, int &b, float w, int nb, int per)
{
    const int s = (r < 0.0f) ? -1 : ((r >= w) ? 1 : 0);
    int nbin = b + s;
    if (per) {
        nbin = (nbin < 1) ? nbin + nb : ((nbin > nb) ? nbin - nb : nbin);
    } else if (nbin < 1 || nbin > nb) {
        return;
    }
    r -= (float)s * w;
    b = nbin;
}

// Bins of the list frames: every exact_every-th build (and the first) bins
// buffer a's FP64 positions exactly and re-derives the FP32 offsets from
// them (rebin_slot_into); the others move each frame by the bin its FP32
// offset has reached, without FP64 arithmetic (GB300 issues FP64 at 1/64 of
// the FP32 rate).  Either way the column counts are accumulated.
__global__ void k_list_rebin(const DevState S, int a)
{
    if (!S.lctl->rebuild) return;
    constexpr int B = kListBins;
    const bool exact = S.lctl->exact_now != 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) S.lctl->body_runs += 1ull;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += gridDim.x * blockDim.x) {
        const DevGeom &G = geom_of(S, i);
        if (exact) {
            rebin_slot_into(S, G, i, S.x[a][i], S.y[a][i], S.z[a][i], S.rad[i], B, a, false);
            continue;
        }
        float4 r = S.rel[a][i];
        int bx, by;
        col_to_bxy(G, S.col[B][i], bx, by);
        int bz = S.iz[B][i];
        reframe(r.x, bx, G.dxf[0], G.n[0], G.per[0]);
        reframe(r.y, by, G.dxf[1], G.n[1], G.per[1]);
        reframe(r.z, bz, G.dxf[2], G.n[2], 0);
        const int c = column_of(G, bx, by);
        S.col[B][i] = c;
        S.iz[B][i] = bz;
        S.rel[a][i] = r;
        atomicAdd(&S.colcnt[c], 1);
    }
}

// Walk every slot's stencil over the column-sorted copies (in sorted order,
// so a warp's lanes share columns) and keep the pairs closer than
// rA + skin (+ a slack covering the FP32 rounding of the test).
__global__ void __launch_bounds__(256) k_list_build(const DevState S, const DevParams P)
{
    if (!S.lctl->rebuild) return;
    constexpr int B = kListBins;
    const int n = S.n;
    const float reach = (float)P.bw + S.lctl->skin;
    unsigned long long over = 0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int i = S.perm[B][t];
        const DevGeom &G = geom_of(S, i);
        int bx, by;
        col_to_bxy(G, S.col[B][i], bx, by);
        const int izi = S.siz[B][t];
        const float4 me = S.srel[B][t];
        const float dxb = G.dxf[0], dyb = G.dxf[1], dzb = G.dxf[2];
        const float lim0 = reach + 4.0e-6f * fmaxf(dxb, fmaxf(dyb, dzb));
        int c = 0;
        visit_sorted(S, G, B, t, bx, by, izi, [&](int u, int dxs, int dys, int dzs, int, int) {
            const float4 q = __ldg(&S.srel[B][u]);
            const float ex = (me.x - q.x) - (float)dxs * dxb;
            const float ey = (me.y - q.y) - (float)dys * dyb;
            const float ez = (me.z - q.z) - (float)dzs * dzb;
            const float r2f = __fmaf_rn(ex, ex, __fmaf_rn(ey, ey, __fmul_rn(ez, ez)));
            const float lim = (me.w + q.w) + lim0;
            if (!(r2f <= lim * lim)) return;
            const unsigned code = (unsigned)(dxs + 1) | ((unsigned)(dys + 1) << 2) | ((unsigned)(dzs + 1) << 4);
            if (c < kNbrCap) S.nbr[(size_t)c * n + i] = (int)((unsigned)__ldg(&S.perm[B][u]) | (code << kNbrShift));
            ++c;
        });
        S.ncnt[i] = c;
        if (c > kNbrCap) ++over;
    }
    if (over) atomicAdd(&S.lctl->overflow, over);
}

// FP32F sphere step over the list: pair math and wall law in FP32 on the
// frozen-frame offsets, FP64 position accumulation and periodic wrap.
__global__ void __launch_bounds__(256) k_list_step(const DevState S, const DevParams P, float dtf, int a)
{
    constexpr int B = kListBins;
    const int b = a ^ 1;
    const int n = S.n;
    const float bwf = (float)P.bw, kf = (float)P.k;
    const float zkf = (float)P.z_k, zbwf = (float)P.z_bw, zgf = (float)P.z_g;
    unsigned dmax = 0u;  // bits of the largest |dt v|^2 (non-negative floats order as integers)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const DevGeom &G = geom_of(S, i);
        const float4 me = S.rel[a][i];
        const int izi = S.iz[B][i];
        const float dxb = G.dxf[0], dyb = G.dxf[1], dzb = G.dxf[2];
        float gx = 0.0f, gy = 0.0f, gz = 0.0f;
        auto pair = [&](const float4 q, float ox, float oy, float oz) {
            const float ex = (me.x - q.x) - ox;
            const float ey = (me.y - q.y) - oy;
            const float ez = (me.z - q.z) - oz;
            const float r2f = __fmaf_rn(ex, ex, __fmaf_rn(ey, ey, __fmul_rn(ez, ez)));
            const float rSf = __fadd_rn(me.w, q.w);
            const float rAf = __fadd_rn(rSf, bwf);
            if (!(r2f < __fmul_rn(rAf, rAf))) return;
            const float inv = rsqrtf(r2f);
            const float rn = __fmul_rn(r2f, inv);
            const float d1 = __fsub_rn(rn, rAf);
            const float F = __fmul_rn(__fmul_rn(__fmul_rn(-kf, d1), d1), __fsub_rn(rn, rSf));
            const float Fi = __fmul_rn(F, inv);
            gx = __fmaf_rn(Fi, ex, gx);
            gy = __fmaf_rn(Fi, ey, gy);
            gz = __fmaf_rn(Fi, ez, gz);
        };
        const int cnt = S.ncnt[i];
        if (cnt <= kNbrCap) {
            auto entry = [&](unsigned e, const float4 q) {
                const unsigned code = e >> kNbrShift;
                pair(q, shift_of(code & 3u, dxb), shift_of((code >> 2) & 3u, dyb), shift_of((code >> 4) & 3u, dzb));
            };
            const int *col = S.nbr + i;
            int k = 0;
            // four entries in flight at a time: the list loads and the
            // neighbour gathers are independent across entries
            for (; k + 4 <= cnt; k += 4) {
                const unsigned e0 = (unsigned)__ldg(col + (size_t)k * n);
                const unsigned e1 = (unsigned)__ldg(col + (size_t)(k + 1) * n);
                const unsigned e2 = (unsigned)__ldg(col + (size_t)(k + 2) * n);
                const unsigned e3 = (unsigned)__ldg(col + (size_t)(k + 3) * n);
                const float4 q0 = __ldg(&S.rel[a][e0 & kSlotMask]);
                const float4 q1 = __ldg(&S.rel[a][e1 & kSlotMask]);
                const float4 q2 = __ldg(&S.rel[a][e2 & kSlotMask]);
                const float4 q3 = __ldg(&S.rel[a][e3 & kSlotMask]);
                entry(e0, q0);
                entry(e1, q1);
                entry(e2, q2);
                entry(e3, q3);
            }
            for (; k < cnt; ++k) {
                const unsigned e = (unsigned)__ldg(col + (size_t)k * n);
                entry(e, __ldg(&S.rel[a][e & kSlotMask]));
            }
        } else {  // list overflow: walk the frozen stencil with the current offsets
            int bx, by;
            col_to_bxy(G, S.col[B][i], bx, by);
            visit_sorted(S, G, B, S.rank[B][i], bx, by, izi, [&](int u, int dxs, int dys, int dzs, int, int) {
                pair(__ldg(&S.rel[a][__ldg(&S.perm[B][u])]), (float)dxs * dxb, (float)dys * dyb,
                     (float)dzs * dzb);
            });
        }
        float dzw;
        if (izi < G.nwz) {
            const float2 c = G.wz[izi];
            dzw = (c.x + me.z) + c.y;
        } else {
            dzw = (float)(S.z[a][i] - P.z_wall);
        }
        const float vx = gx, vy = gy, vz = gz + wall_law32(dzw, me.w, zkf, zbwf, zgf);
        const float ix = dtf * vx, iy = dtf * vy, iz = dtf * vz;
        double nx = S.x[a][i] + f2d_int(ix);
        double ny = S.y[a][i] + f2d_int(iy);
        const double nz = S.z[a][i] + f2d_int(iz);
        if (G.per[0] && (dkey(nx) < dkey(G.plo[0]) || dkey(nx) >= dkey(G.phi[0])))
            nx = wrap1(nx, G.plo[0], G.phi[0], G.len[0]);
        if (G.per[1] && (dkey(ny) < dkey(G.plo[1]) || dkey(ny) >= dkey(G.phi[1])))
            ny = wrap1(ny, G.plo[1], G.phi[1], G.len[1]);
        S.x[b][i] = nx;
        S.y[b][i] = ny;
        S.z[b][i] = nz;
        S.rel[b][i] = make_float4(me.x + ix, me.y + iy, me.z + iz, me.w);
        S.vxf[i] = vx;
        S.vyf[i] = vy;
        S.vzf[i] = vz;
        if (dkey(nz) < dkey(G.plo[2]) || dkey(nz) >= dkey(G.phi[2])) atomicAdd(&S.cnt->out_of_domain, 1ULL);
        const float d2 = __fmaf_rn(ix, ix, __fmaf_rn(iy, iy, __fmul_rn(iz, iz)));
        if (!isfinite(d2)) atomicAdd(&S.cnt->nonfinite, 1ULL);
        dmax = max(dmax, isfinite(d2) ? __float_as_uint(d2) : 0x7f800000u);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dmax = max(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
    if ((threadIdx.x & 31) == 0 && dmax) atomicMax(&S.lctl->maxd2_bits, dmax);
}

}  // namespace

int launch_list_decide(const DevState &S, unsigned long long cond, int use_cond, cudaStream_t st)
{
    k_list_decide<<<1, 1, 0, st>>>(S.lctl, (cudaGraphConditionalHandle)cond, use_cond);
    return 1;
}

int launch_list_rebuild(const DevState &S, const DevParams &P, int a, int *scan_scratch, int grid, int block,
                        cudaStream_t st)
{
    const int *gate = &S.lctl->rebuild;
    k_list_rebin<<<grid, block, 0, st>>>(S, a);
    int k = 1 + launch_rebuild(S, kListBins, scan_scratch, grid, block, st, a, gate);
    k_list_build<<<grid, block, 0, st>>>(S, P);
    return k + 1;
}

int launch_list_step(const DevState &S, const DevParams &P, double dt, int a, int grid, int block,
                     cudaStream_t st)
{
    k_list_step<<<grid, block, 0, st>>>(S, P, (float)dt, a);
    return 1;
}

}  // namespace bmxg
