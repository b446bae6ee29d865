// k_list.cu -- FP32F sphere step over a neighbour list with a skin.
//
// The force acts only on pairs closer than rA = r_i + r_j + bw
// (maxInteractionDistance and the gate r^2 <= (r_lm - 1e-15)^2,
// bmx_cell_interaction_K.H:23-40, bmx_pc_interaction.cpp:212).  When
// rA + skin is at most the smallest bin width, any pair that close sits in
// neighbouring bins, so the reference's stencil list holds it whatever the
// binning is.  The list built here holds every pair closer than rA + skin
// at build time; while no pair's separation has changed by the skin since,
// it still holds every pair closer than rA.  The pair set of a step is
// therefore the reference's; only the FP32 rounding of the pair math (the
// precision form) differs from it.
//
// Between builds the bins stay frozen (buffer kListBins) and the FP32
// offsets advance in the frozen frame, while the FP64 positions accumulate
// and wrap periodically every step as in the reference.  A build moves
// every frame to the bin its offset has reached (every kListExactEvery-th
// build re-bins exactly from the FP64 positions instead, which also bounds
// the FP32 drift of the offsets), rebuilds the cell lists and walks the
// stencil once.  The bins need not be the reference's here: with
// rA + skin within a bin width, any binning finds the same pairs.
// k_list_decide bounds the separation change of every pair from the spread
// of each step's increments and asks for a build when the bound reaches the
// skin (or after max_age steps); inside a CUDA graph the build kernels sit
// in a conditional node that the decision switches, so a step without a
// build launches two kernels.
//
// Roofline: the step kernel streams the slot state (FP64 positions in and
// out, FP32 offsets in and out, FP32 velocities out) and the list; the
// neighbour offsets it gathers are L2-resident.  HBM bound, no contraction.
#include <algorithm>

#include "bmxg_stencil.cuh"

namespace bmxg {

namespace {

constexpr unsigned kSlotMask = (1u << kNbrShift) - 1u;

// Order-preserving unsigned key of a float (and back): atomicMin / atomicMax
// on the keys order the floats.
__device__ __forceinline__ unsigned fkey(float f)
{
    const unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__device__ __forceinline__ float funkey(unsigned k)
{
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

constexpr unsigned kKeyPosInf = 0xff800000u;  // fkey(+inf)
constexpr unsigned kKeyNegInf = 0x007fffffu;  // fkey(-inf)

// The bound: for any pair, the separation change since the build is, per
// component, at most the sum over steps of the spread (largest minus
// smallest) of that step's increments; its length at most the length of
// those sums.  Unlike twice the largest displacement, it does not count a
// drift common to all slots (here: the rise of the slots below the growth
// surface).  Each step adds eps_step per component for the FP32 rounding of
// the offset updates.
// It also clears the per-step counters (no memset nodes in the step).
__global__ void k_list_decide(ListCtl *c, DevCounters *cnt, cudaGraphConditionalHandle h, int use_h)
{
    cnt->out_of_domain = 0ull;
    cnt->edge_ghost = 0ull;
    cnt->pairs = 0ull;
    cnt->bond_repairs = 0ull;
    cnt->moved = 0ull;
    float r2 = 0.0f;
    float rg[3];
    for (int k = 0; k < 3; ++k) {
        const unsigned lo = c->inc_min[k], hi = c->inc_max[k];
        // no slot reported (empty state): no spread
        const float spread = (hi >= lo) ? (funkey(hi) - funkey(lo)) : 0.0f;
        rg[k] = c->range[k] + spread * 1.000001f + c->eps_step;
        r2 += rg[k] * rg[k];
        c->inc_min[k] = kKeyPosInf;
        c->inc_max[k] = kKeyNegInf;
    }
    const float acc = sqrtf(r2);
    const int age = c->age + 1;
    const bool rb = c->force != 0 || !(acc <= c->skin) || age > c->max_age;
    if (rb) {
        // force 1: state changed, bins unknown (exact); force 2: the list bins
        // are already the exact bins of the positions (no FP64 re-binning)
        c->exact_now = (c->force == 1 || (c->force == 0 && c->builds % c->exact_every == 0)) ? 1 : 0;
        for (int k = 0; k < 3; ++k) c->range[k] = 0.0f;
        c->acc = 0.0f;
        c->age = 0;
        c->force = 0;
        c->builds += 1;
        c->overflow = 0ull;
    } else {
        for (int k = 0; k < 3; ++k) c->range[k] = rg[k];
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

__device__ __forceinline__ int cell_of(const DevGeom &G, int bx, int by, int bz)
{
    return G.cell_base + ((bx - 1) * G.n[1] + (by - 1)) * G.n[2] + (bz - 1);
}

// Bins of the list frames: every exact_every-th build (and the first) bins
// buffer a's FP64 positions exactly and re-derives the FP32 offsets from
// them (rebin_slot_into); the others move each frame by the bin its FP32
// offset has reached, without FP64 arithmetic (GB300 issues FP64 at 1/64 of
// the FP32 rate).  Either way the 3D cell counts are accumulated.
__global__ void k_list_rebin(const DevState S, int a)
{
    if (!S.lctl->rebuild) return;
    constexpr int B = kListBins;
    const bool exact = S.lctl->exact_now != 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) S.lctl->body_runs += 1ull;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += gridDim.x * blockDim.x) {
        const DevGeom &G = geom_of(S, i);
        int bx, by, bz;
        if (exact) {
            // (the column counters are the per-step paths'; the list counts cells)
            rebin_slot_into(S, G, i, S.x[a][i], S.y[a][i], S.z[a][i], S.rad[i], B, a, false, false);
            col_to_bxy(G, S.col[B][i], bx, by);
            bz = S.iz[B][i];
        } else {
            float4 r = S.rel[a][i];
            col_to_bxy(G, S.col[B][i], bx, by);
            bz = S.iz[B][i];
            reframe(r.x, bx, G.dxf[0], G.n[0], G.per[0]);
            reframe(r.y, by, G.dxf[1], G.n[1], G.per[1]);
            reframe(r.z, bz, G.dxf[2], G.n[2], 0);
            S.col[B][i] = column_of(G, bx, by);
            S.iz[B][i] = bz;
            S.rel[a][i] = r;
        }
        atomicAdd(&S.cellcnt[cell_of(G, bx, by, bz)], 1);
    }
}

// counting sort into the cells (arrival order from the atomics)
__global__ void k_list_scatter(const DevState S)
{
    if (!S.lctl->rebuild) return;
    constexpr int B = kListBins;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += gridDim.x * blockDim.x) {
        const DevGeom &G = geom_of(S, i);
        int bx, by;
        col_to_bxy(G, S.col[B][i], bx, by);
        const int c = cell_of(G, bx, by, S.iz[B][i]);
        const int r = atomicSub(&S.cellcnt[c], 1) - 1;  // leaves cellcnt at zero
        const int t = S.cellstart[c] + r;
        if (t >= 0 && t < S.n) S.tmp[t] = i;
        else atomicAdd(&S.cnt->bad_index, 1ULL);
    }
}

// deterministic order inside a cell (ascending original index), and the
// sorted copies the build walks: offsets, z bin, slot, and each slot's rank
__global__ void k_list_canon(const DevState S, int a)
{
    if (!S.lctl->rebuild) return;
    constexpr int B = kListBins;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += gridDim.x * blockDim.x) {
        const DevGeom &G = geom_of(S, i);
        int bx, by;
        col_to_bxy(G, S.col[B][i], bx, by);
        const int bz = S.iz[B][i];
        const int c = cell_of(G, bx, by, bz);
        const int s0 = max(S.cellstart[c], 0), s1 = min(S.cellstart[c + 1], S.n);
        const int oi = S.orig[i];
        int rank = 0;
        for (int t = s0; t < s1; ++t) {
            const int j = S.tmp[t];
            if ((unsigned)j < (unsigned)S.n) rank += (S.orig[j] < oi);
        }
        const int t = s0 + rank;
        if (t >= s1) {  // i is not among its cell's members: inconsistent counts
            atomicAdd(&S.cnt->bad_index, 1ULL);
            continue;
        }
        S.perm[B][t] = i;
        S.srel[B][t] = S.rel[a][i];
        S.siz[B][t] = bz;
        S.rank[B][i] = t;
    }
}

// Visit the slots of the 3 x 3 neighbour columns of bin (bx, by), z bins
// izi - 1 .. izi + 1 (periodic images included), as contiguous cell ranges
// of the sorted copies.  f(u, dxs, dys, dzs): sorted position and the bin
// shift of the neighbour relative to (bx, by, izi); the slot's own sorted
// position self_t is skipped.  (One loop per column over its three z cells
// keeps the lanes of a warp together better than a loop per cell; a
// candidate's z bin follows from the cell boundaries inside the range.)
template <class F>
__device__ __forceinline__ void visit_cells(const DevState &S, const DevGeom &G, int self_t, int bx, int by, int izi,
                                            F &&f)
{
    const int *__restrict__ cs = S.cellstart;
    const int nz = G.n[2];
    const int z0 = max(izi - 1, 1), z1 = min(izi + 1, nz);
    for (int dxs = -1; dxs <= 1; ++dxs) {
        int sx = bx + dxs;
        if (sx < 1 || sx > G.n[0]) {
            if (!G.per[0]) continue;
            sx += (sx < 1) ? G.n[0] : -G.n[0];
        }
        for (int dys = -1; dys <= 1; ++dys) {
            int sy = by + dys;
            if (sy < 1 || sy > G.n[1]) {
                if (!G.per[1]) continue;
                sy += (sy < 1) ? G.n[1] : -G.n[1];
            }
            const int cb = G.cell_base + ((sx - 1) * G.n[1] + (sy - 1)) * nz;
            const int hi = __ldg(&cs[cb + z1]);
            // z bin of a candidate from the cell boundaries inside the range
            const int m1 = __ldg(&cs[cb + z0]), m2 = (z1 > z0) ? __ldg(&cs[cb + z0 + 1]) : hi;
            const int dz0 = z0 - izi;
            for (int u = __ldg(&cs[cb + z0 - 1]); u < hi; ++u) {
                if (u == self_t) continue;
                f(u, dxs, dys, dz0 + (u >= m1) + (u >= m2));
            }
        }
    }
}

// List build: every slot (in sorted order, so a warp's lanes share cells)
// keeps the neighbours closer than rA + skin (+ a slack covering the FP32
// rounding of the test), and its packed metadata: z bin, edge flags (x or y
// bin on a periodic face, z bin at a closed face) and list length.
__global__ void __launch_bounds__(kListBuildBlock) k_list_build(const DevState S, const DevParams P)
{
    if (!S.lctl->rebuild) return;
    constexpr int B = kListBins;
    const int n = S.n;
    const float reach = P.bw32 + S.lctl->skin;
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
        int4 rec = make_int4(0, 0, 0, 0);
        visit_cells(S, G, t, bx, by, izi, [&](int u, int dxs, int dys, int dzs) {
            const float4 q = __ldg(&S.srel[B][u]);
            const float ex = (me.x - q.x) - (float)dxs * dxb;
            const float ey = (me.y - q.y) - (float)dys * dyb;
            const float ez = (me.z - q.z) - (dzs == 0 ? 0.0f : (dzs > 0 ? dzb : -dzb));
            const float r2f = __fmaf_rn(ex, ex, __fmaf_rn(ey, ey, __fmul_rn(ez, ez)));
            const float lim = (me.w + q.w) + lim0;
            if (!(r2f <= lim * lim)) return;
            const unsigned code = (unsigned)(dxs & 3) | ((unsigned)(dys & 3) << 2) | ((unsigned)(dzs & 3) << 4);
            const int e = (int)((unsigned)__ldg(&S.perm[B][u]) | (code << kNbrShift));
            if (c == 0) rec.y = e;
            else if (c == 1) rec.z = e;
            else if (c == 2) rec.w = e;
            else if (c < kNbrCap) S.nbr[(size_t)(c - kNbrInline) * n + i] = e;
            ++c;
        });
        const int edge = ((G.per[0] && (bx == 1 || bx == G.n[0])) ? 1 : 0) |
                         ((G.per[1] && (by == 1 || by == G.n[1])) ? 2 : 0) | ((izi == 1 || izi == G.n[2]) ? 4 : 0);
        rec.x = izi | (edge << 16) | (min(c, 255) << 20);
        S.lrec[i] = rec;
        if (c > kNbrCap) ++over;
    }
    if (over) atomicAdd(&S.lctl->overflow, over);
}

// FP32F sphere step over the list: pair math and wall law in FP32 on the
// frozen-frame offsets, FP64 position accumulation; the periodic wrap and
// the domain test (FP64 compares) only run for slots whose frozen bin is on
// a face, the only ones that can cross it before the next build.
// Each block takes a contiguous chunk of slots, so a thread's colony is
// found by one binary search and then by stepping forward from the last one.
// The list metadata and the first entries come in one 16-byte record.
// (128, 12): 40 registers without spills, twelve blocks of four warps per SM;
// the kernel is latency bound and wants every resident warp (128-thread
// blocks: 92.4 us against 94.3 us with 256 threads in six blocks, the block
// scheduler balancing the uneven lists at a finer grain)
__global__ void __launch_bounds__(kListStepBlock, 12) k_list_step(const DevState S, const DevParams P, float dtf, int a, int chunk)
{
    constexpr int B = kListBins;
    const int b = a ^ 1;
    const int n = S.n;
    const float bwf = P.bw32, kf = P.k32;
    const float zkf = P.z_k32, zbwf = P.z_bw32, zgf = P.z_g32;
    const float4 *__restrict__ rel_a = S.rel[a];
    const int *__restrict__ nbr = S.nbr;
    // smallest and largest increment per component (order-preserving keys),
    // per warp in shared memory: reduced over the warp after each pass, so
    // that no register holds them through the list walk
    __shared__ unsigned wmin[32][3], wmax[32][3];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane < 3) {
        wmin[w][lane] = kKeyPosInf;
        wmax[w][lane] = kKeyNegInf;
    }
    __syncwarp();
    const int i0 = blockIdx.x * chunk;
    const int i1 = min(i0 + chunk, n);
    int colony = (i0 + (int)threadIdx.x < i1) ? colony_of(S.cbase, S.ncol, i0 + threadIdx.x) : 0;
    for (int base = i0; base < i1; base += blockDim.x) {  // same trip count for every thread
        const int i = base + threadIdx.x;
        unsigned lo0 = kKeyPosInf, lo1 = kKeyPosInf, lo2 = kKeyPosInf;
        unsigned hi0 = kKeyNegInf, hi1 = kKeyNegInf, hi2 = kKeyNegInf;
        if (i < i1) {
            while (colony + 1 < S.ncol && __ldg(&S.cbase[colony + 1]) <= i) ++colony;
            const DevGeom &G = S.geoms[colony];
            const float4 me = rel_a[i];
            const int4 rec = __ldg(&S.lrec[i]);
            const int meta = rec.x;
            const int izi = meta & 0xffff;
            const int edge = (meta >> 16) & 7;
            const int cnt = meta >> 20;
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
            if (cnt <= kNbrCap) {
                auto entry = [&](unsigned e, const float4 q) {
                    // signed 2-bit shifts at bits 26-27, 28-29, 30-31
                    pair(q, (float)((int)(e << 4) >> 30) * dxb, (float)((int)(e << 2) >> 30) * dyb,
                         (float)((int)e >> 30) * dzb);
                };
                // the first entries came with the metadata: their gathers go out
                // together, one round trip for the typical short list
                const float4 z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                const float4 p0 = (cnt > 0) ? __ldg(&rel_a[(unsigned)rec.y & kSlotMask]) : z4;
                const float4 p1 = (cnt > 1) ? __ldg(&rel_a[(unsigned)rec.z & kSlotMask]) : z4;
                const float4 p2 = (cnt > 2) ? __ldg(&rel_a[(unsigned)rec.w & kSlotMask]) : z4;
                if (cnt > 0) entry((unsigned)rec.y, p0);
                if (cnt > 1) entry((unsigned)rec.z, p1);
                if (cnt > 2) entry((unsigned)rec.w, p2);
                const int *col = nbr + i;  // entry k in plane k - kNbrInline
                int k = kNbrInline;
                // four entries in flight at a time: the list loads and the
                // neighbour gathers are independent across entries
                for (; k + 4 <= cnt; k += 4) {
                    const unsigned e0 = (unsigned)__ldg(col + (size_t)(k - kNbrInline) * n);
                    const unsigned e1 = (unsigned)__ldg(col + (size_t)(k + 1 - kNbrInline) * n);
                    const unsigned e2 = (unsigned)__ldg(col + (size_t)(k + 2 - kNbrInline) * n);
                    const unsigned e3 = (unsigned)__ldg(col + (size_t)(k + 3 - kNbrInline) * n);
                    const float4 q0 = __ldg(&rel_a[e0 & kSlotMask]);
                    const float4 q1 = __ldg(&rel_a[e1 & kSlotMask]);
                    const float4 q2 = __ldg(&rel_a[e2 & kSlotMask]);
                    const float4 q3 = __ldg(&rel_a[e3 & kSlotMask]);
                    entry(e0, q0);
                    entry(e1, q1);
                    entry(e2, q2);
                    entry(e3, q3);
                }
                for (; k < cnt; ++k) {
                    const unsigned e = (unsigned)__ldg(col + (size_t)(k - kNbrInline) * n);
                    entry(e, __ldg(&rel_a[e & kSlotMask]));
                }
            } else {  // list overflow: walk the frozen cells with the current offsets
                int bx, by;
                col_to_bxy(G, S.col[B][i], bx, by);
                visit_cells(S, G, S.rank[B][i], bx, by, izi, [&](int u, int dxs, int dys, int dzs) {
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
            if (edge) {
                if (edge & 1) nx = wrap1(nx, G.plo[0], G.phi[0], G.len[0]);
                if (edge & 2) ny = wrap1(ny, G.plo[1], G.phi[1], G.len[1]);
                if ((edge & 4) && !(nz >= G.plo[2] && nz < G.phi[2])) atomicAdd(&S.cnt->out_of_domain, 1ULL);
            }
            S.x[b][i] = nx;
            S.y[b][i] = ny;
            S.z[b][i] = nz;
            S.rel[b][i] = make_float4(me.x + ix, me.y + iy, me.z + iz, me.w);
            S.vxf[i] = vx;
            S.vyf[i] = vy;
            S.vzf[i] = vz;
            lo0 = hi0 = fkey(ix);
            lo1 = hi1 = fkey(iy);
            lo2 = hi2 = fkey(iz);
            if (!isfinite(ix + iy + iz)) {
                atomicAdd(&S.cnt->nonfinite, 1ULL);
                lo0 = 0u;  // spreads the bound: the next step rebuilds
                hi0 = 0xffffffffu;
            }
        }
        lo0 = __reduce_min_sync(0xffffffffu, lo0);
        hi0 = __reduce_max_sync(0xffffffffu, hi0);
        lo1 = __reduce_min_sync(0xffffffffu, lo1);
        hi1 = __reduce_max_sync(0xffffffffu, hi1);
        lo2 = __reduce_min_sync(0xffffffffu, lo2);
        hi2 = __reduce_max_sync(0xffffffffu, hi2);
        if (lane == 0) {
            wmin[w][0] = min(wmin[w][0], lo0);
            wmax[w][0] = max(wmax[w][0], hi0);
            wmin[w][1] = min(wmin[w][1], lo1);
            wmax[w][1] = max(wmax[w][1], hi1);
            wmin[w][2] = min(wmin[w][2], lo2);
            wmax[w][2] = max(wmax[w][2], hi2);
        }
    }
    // then over the block: six atomics per block, not per warp (updates of
    // one address serialise in its L2 slice)
    __syncthreads();
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        unsigned lo = kKeyPosInf, hi = kKeyNegInf;
        for (int v = 0; v < nw; ++v) {
            lo = min(lo, wmin[v][k]);
            hi = max(hi, wmax[v][k]);
        }
        if (hi >= lo) {
            atomicMin(&S.lctl->inc_min[k], lo);
            atomicMax(&S.lctl->inc_max[k], hi);
        }
    }
}

}  // namespace

int launch_list_decide(const DevState &S, unsigned long long cond, int use_cond, cudaStream_t st)
{
    k_list_decide<<<1, 1, 0, st>>>(S.lctl, S.cnt, (cudaGraphConditionalHandle)cond, use_cond);
    return 1;
}

int launch_list_rebuild(const DevState &S, const DevParams &P, int a, int *scan_scratch, int grid, int block,
                        cudaStream_t st)
{
    const int *gate = &S.lctl->rebuild;
    k_list_rebin<<<grid, block, 0, st>>>(S, a);
    int k = 1 + launch_scan(S.cellcnt, S.cellstart, S.ncells_total, scan_scratch, st, gate);
    k_list_scatter<<<grid, block, 0, st>>>(S);
    k_list_canon<<<grid, block, 0, st>>>(S, a);
    // the build: one slot per thread in 128-thread blocks (the stencil walks
    // differ in length from slot to slot; small blocks on a grid of every
    // slot let the scheduler balance them: 150.0 -> 145.7 us per whole step
    // against 256-thread blocks striding over one wave)
    k_list_build<<<(S.n + kListBuildBlock - 1) / kListBuildBlock, kListBuildBlock, 0, st>>>(S, P);
    return k + 3;
}

int launch_list_step(const DevState &S, const DevParams &P, double dt, int a, int grid, int block,
                     cudaStream_t st)
{
    // two passes of the block per chunk: short enough that the block
    // scheduler evens out the uneven list lengths of the colonies (one wave
    // of long chunks ends on its slowest block), long enough to amortise the
    // colony search and the block's reduction of the increment spreads.  One
    // pass when two would leave fewer than four waves of twelve blocks per SM
    // (grid = the SM count): small states need the blocks more.
    const int two = (S.n + 2 * block - 1) / (2 * block);
    const int chunk = (two >= 4 * 12 * grid) ? 2 * block : block;
    k_list_step<<<(S.n + chunk - 1) / chunk, block, 0, st>>>(S, P, (float)dt, a, chunk);
    return 1;
}

}  // namespace bmxg
