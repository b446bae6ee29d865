// k_sphere.cu -- fused sphere step: force gather over the neighbour stencil,
// growth-surface force, overdamped update, periodic wrap and rebin, one pass.
//
// Replaces, for YEAST-only states, the force lambda of
// src/des/bmx_pc_interaction.cpp:170-279 (evaluateForce's sphere branch,
// src/chemistry/bmx_cell_interaction_K.H:243-276, and evaluateSurfaceForce's
// sphere branch, :1009-1030) and the update lambda (:311-436), followed by
// the periodic wrap of the trailing Redistribute (:485-486).
//
// Forms:
//  FP64  (plain, k_sphere64) every pair that can pass the reference's cutoff
//        test is evaluated in FP64 with the reference's operation order (this
//        file is compiled with -fmad=false), accumulated in list order: the
//        result is bit-identical to the host oracle.  Pairs are first
//        screened in FP32 from the bin-relative offsets with an absolute
//        slack that bounds the FP32 error, so only pairs that are certainly
//        beyond the cutoff skip the FP64 test.
//  FP32F (precision form, k_sphere32) pair math and wall law in FP32 on
//        FP64-differenced bin-relative offsets; the position accumulation
//        stays FP64.  GB300 issues FP64 at 1/64 of the FP32 rate, so the
//        per-particle epilogue avoids FP64 too: the bin-relative offsets are
//        advanced in FP32 and re-derived exactly from the FP64 position
//        (exact FP64 re-binning) every kResyncEvery-th step and whenever a
//        particle comes within a guard band of a bin face, where its bin
//        might change.  Away from the faces the FP64 bin cannot change, so
//        the neighbour lists stay exactly the reference's.
// Roofline: HBM / L2 bound gather; no dense contraction, so no tensor cores.
#include "bmxg_stencil.cuh"

namespace bmxg {

namespace {

// The FP64 pair term of slot i (at xi, yi, zi, radius ri, colony geometry
// G) from neighbour j under image shift (sx, sy), in the reference's operation
// order: false when the pair is not in the neighbour list or beyond the
// cutoff, else the three products F u_x, F u_y, F u_z that the gather adds.
__device__ __forceinline__ bool sphere_term64(const DevState &S, const DevGeom &G, const DevParams &P, int a,
                                              double xi, double yi, double zi, double ri, int j, int sx, int sy,
                                              double *t)
{
    const double xj = sx ? S.x[a][j] + (double)sx * G.len[0] : S.x[a][j];
    const double yj = sy ? S.y[a][j] + (double)sy * G.len[1] : S.y[a][j];
    const double dx = xi - xj, dy = yi - yj, dz = zi - S.z[a][j];
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (!G.nbh_trivial && !(r2 <= P.nbh)) return false;  // not in the neighbour list
    const double rj = S.rad[j];
    const double rlm = ri + rj + P.bw;                     // maxInteractionDistance
    if (!(r2 <= (rlm - kSmall) * (rlm - kSmall))) return false;
    const double rS = ri + rj;
    const double rA = rS + P.bw;
    const double rn = sqrt(r2);
    const double ux = dx / rn, uy = dy / rn, uz = dz / rn;
    const double F = (rn < rA) ? -P.k * (rn - rA) * (rn - rA) * (rn - rS) : 0.0;
    t[0] = F * ux;
    t[1] = F * uy;
    t[2] = F * uz;
    return true;
}

// FP64 plain step.  Each thread walks its slot's stencil and screens the
// candidates in FP32 (FP32 and integer work); the few that can pass the
// cutoff (about 1.3 per slot on the colonies) are staged in shared memory,
// and the block then evaluates its slots' staged pairs together, one per
// thread, so that the FP64 gate, square root and divisions run in full warps
// (GB300 issues FP64 at 2 lanes per clock per SM whatever the mask: a thread
// walking its own candidates keeps 8 of 32 lanes busy in those instructions),
// and a warp whose share of a round is empty skips it.  Each slot then adds
// its pairs' terms in walk order -- the same FP64 values in the same order as
// a walk that evaluates each pair when it meets it, so the result stays
// bit-identical to the oracle.  A slot with more than kStage64 staged
// candidates evaluates them itself, in order, as it walks.
constexpr int kStage64 = 16;

// dynamic shared memory of k_sphere64 for a block of `block` threads
__host__ __device__ constexpr size_t sphere64_smem(int block)
{
    return (size_t)block * (kStage64 * sizeof(int2) + 4 * sizeof(double) + 3 * sizeof(double) + 4 * sizeof(int)) +
           2 * 32 * sizeof(int);
}

template <bool SORTED>
__global__ void __launch_bounds__(256) k_sphere64(const DevState S, const DevParams P, double dt, int a)
{
    // per thread: its staged candidates (j, image code); its slot's position,
    // radius, colony and run of staged pairs (for the block's evaluation);
    // one round's terms and gate results
    extern __shared__ __align__(16) unsigned char sm64[];
    const int B = blockDim.x, tid = threadIdx.x;
    const int lane = tid & 31, w = tid >> 5, nw = B >> 5;
    int2 *stage = reinterpret_cast<int2 *>(sm64);
    double *opos = reinterpret_cast<double *>(stage + (size_t)B * kStage64);  // 4 per thread: x, y, z, r
    double *term = opos + 4 * B;                                               // 3 per thread
    int *ocol = reinterpret_cast<int *>(term + 3 * B);
    int *orun = ocol + B;   // first staged pair of the slot in the block's run
    int *olen = orun + B;   // its staged pairs
    int *opass = olen + B;  // the round's gate result per thread
    int *wsum = opass + B;  // per warp: staged pairs, then their exclusive scan
    const int b = a ^ 1;
    const float bwf = (float)P.bw;  // once per thread: a conversion is an FP64-pipe instruction
    for (int base = blockIdx.x * B; base < S.n; base += gridDim.x * B) {
        const int i = base + tid;
        const bool act = i < S.n;
        double xi = 0.0, yi = 0.0, zi = 0.0, ri = 0.0;
        double fx = 0.0, fy = 0.0, fz = 0.0;
        int col = 0, cnt = 0;
        if (act) {
            col = colony_of(S.cbase, S.ncol, i);
            const DevGeom &G = S.geoms[col];
            int bx, by;
            col_to_bxy(G, S.col[a][i], bx, by);
            const int izi = S.iz[a][i];
            xi = S.x[a][i];
            yi = S.y[a][i];
            zi = S.z[a][i];
            ri = S.rad[i];
            const float4 me = S.rel[a][i];
            const float dxb = G.dxf[0], dyb = G.dxf[1], dzb = G.dxf[2];
            // absolute slack bounding the FP32 distance error (offsets + bin widths)
            const float slack = 8.0f * 1.1920929e-7f * fmaxf(dxb, fmaxf(dyb, dzb));
            int2 *mine = stage + (size_t)tid * kStage64;
            auto eval = [&](int j, int sx, int sy) {
                double t[3];
                if (sphere_term64(S, G, P, a, xi, yi, zi, ri, j, sx, sy, t)) {
                    fx += t[0];
                    fy += t[1];
                    fz += t[2];
                }
            };
            walk<SORTED>(S, G, a, i, bx, by, izi, [&](const float4 q, auto slot, int dxs, int dys, int dzs, int sx,
                                                      int sy) {
                const float ex = (me.x - q.x) - (float)dxs * dxb;
                const float ey = (me.y - q.y) - (float)dys * dyb;
                const float ez = (me.z - q.z) - (float)dzs * dzb;
                const float r2f = __fmaf_rn(ex, ex, __fmaf_rn(ey, ey, __fmul_rn(ez, ez)));
                const float lim = __fadd_rn(__fadd_rn(__fadd_rn(me.w, q.w), bwf), slack);
                if (r2f > __fmul_rn(lim, lim)) return;
                const int j = slot();
                if (cnt < kStage64) {
                    mine[cnt] = make_int2(j, (sx + 1) * 3 + (sy + 1));
                } else {
                    if (cnt == kStage64)  // too many for the stage: the staged ones first, in order
                        for (int k = 0; k < kStage64; ++k) eval(mine[k].x, mine[k].y / 3 - 1, mine[k].y % 3 - 1);
                    eval(j, sx, sy);
                }
                ++cnt;
            });
        }
        // the block's run of staged pairs: slot by slot in thread order
        const int xl = (cnt <= kStage64) ? cnt : 0;
        int xo = xl;
        for (int d = 1; d < 32; d <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, xo, d);
            if (lane >= d) xo += v;
        }
        if (lane == 31) wsum[w] = xo;
        opos[4 * tid] = xi;
        opos[4 * tid + 1] = yi;
        opos[4 * tid + 2] = zi;
        opos[4 * tid + 3] = ri;
        ocol[tid] = col;
        olen[tid] = xl;
        __syncthreads();
        if (tid == 0) {
            int run = 0;
            for (int v = 0; v < nw; ++v) {
                const int c = wsum[v];
                wsum[32 + v] = run;
                run += c;
            }
            wsum[31] = run;  // (nw <= 8: slot 31 is free) the block's total
        }
        __syncthreads();
        const int xt = wsum[31];
        xo += wsum[32 + w] - xl;
        orun[tid] = xo;
        __syncthreads();
        for (int t0 = 0; t0 < xt; t0 += B) {
            const int t = t0 + tid;
            int pass = 0;
            double tt[3] = {0.0, 0.0, 0.0};
            if (t0 + 32 * w < xt) {  // a warp with no pair in this round skips it
                if (t < xt) {
                    int o = 0;  // the slot that owns pair t: the last thread whose run starts at or before t
                    for (int s2 = 1 << (31 - __clz(max(B - 1, 1))); s2 >= 1; s2 >>= 1)
                        if (o + s2 < B && orun[o + s2] <= t) o += s2;
                    const int2 e = stage[(size_t)o * kStage64 + (t - orun[o])];
                    pass = sphere_term64(S, S.geoms[ocol[o]], P, a, opos[4 * o], opos[4 * o + 1], opos[4 * o + 2],
                                         opos[4 * o + 3], e.x, e.y / 3 - 1, e.y % 3 - 1, tt)
                               ? 1
                               : 0;
                }
            }
            term[3 * tid] = tt[0];
            term[3 * tid + 1] = tt[1];
            term[3 * tid + 2] = tt[2];
            opass[tid] = pass;
            __syncthreads();
            const int k1 = min(xo + xl, t0 + B);
            for (int k = max(xo, t0); k < k1; ++k) {
                if (!opass[k - t0]) continue;
                fx += term[3 * (k - t0)];
                fy += term[3 * (k - t0) + 1];
                fz += term[3 * (k - t0) + 2];
            }
            __syncthreads();
        }
        if (act) {
            const DevGeom &G = S.geoms[col];
            // evaluateSurfaceForce, sphere branch: vcom = (0, 0, wall), vrot = 0
            const double vx = fx + 0.0;
            const double vy = fy + 0.0;
            const double vz = fz + wall_law(zi, ri, P);
            double nx = xi + dt * vx;
            double ny = yi + dt * vy;
            const double nz = zi + dt * vz;
            if (G.per[0]) nx = wrap1(nx, G.plo[0], G.phi[0], G.len[0]);
            if (G.per[1]) ny = wrap1(ny, G.plo[1], G.phi[1], G.len[1]);
            S.x[b][i] = nx;
            S.y[b][i] = ny;
            S.z[b][i] = nz;
            S.vx[i] = vx;
            S.vy[i] = vy;
            S.vz[i] = vz;
            rebin_slot(S, G, i, nx, ny, nz, ri, b);
        }
        __syncthreads();  // the next pass reuses the stage and the slot records
    }
}

template <bool SORTED>
__global__ void __launch_bounds__(256, 5) k_sphere32(const DevState S, const DevParams P, float dtf, int a,
                                                  int resync)
{
    const int b = a ^ 1;
    // the FP32 roundings come from the host (a conversion is an FP64-pipe
    // instruction, and threads without a slot would issue them too)
    const float bwf = P.bw32, kf = P.k32;
    const float zkf = P.z_k32, zbwf = P.z_bw32, zgf = P.z_g32;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += gridDim.x * blockDim.x) {
        const DevGeom &G = geom_of(S, i);
        const int col = S.col[a][i];
        int bx, by;
        col_to_bxy(G, col, bx, by);
        const int izi = S.iz[a][i];
        const float4 me = S.rel[a][i];
        const float dxb = G.dxf[0], dyb = G.dxf[1], dzb = G.dxf[2];
        float gx = 0.0f, gy = 0.0f, gz = 0.0f;
        walk<SORTED>(S, G, a, i, bx, by, izi, [&](const float4 q, auto slot, int dxs, int dys, int dzs, int sx, int sy) {
            const float ex = (me.x - q.x) - (float)dxs * dxb;
            const float ey = (me.y - q.y) - (float)dys * dyb;
            const float ez = (me.z - q.z) - (float)dzs * dzb;
            const float r2f = __fmaf_rn(ex, ex, __fmaf_rn(ey, ey, __fmul_rn(ez, ez)));
            const float rAf = __fadd_rn(__fadd_rn(me.w, q.w), bwf);
            if (!(r2f < __fmul_rn(rAf, rAf))) return;
            if (!G.nbh_trivial) {  // BMXCheckPair, exactly (FP64)
                const int j = slot();
                const double xj = sx ? S.x[a][j] + (double)sx * G.len[0] : S.x[a][j];
                const double yj = sy ? S.y[a][j] + (double)sy * G.len[1] : S.y[a][j];
                const double dx = S.x[a][i] - xj, dy = S.y[a][i] - yj, dz = S.z[a][i] - S.z[a][j];
                if (!(dx * dx + dy * dy + dz * dz <= P.nbh)) return;
            }
            const float inv = rsqrtf(r2f);
            const float rn = __fmul_rn(r2f, inv);
            const float rSf = __fadd_rn(me.w, q.w);
            const float d1 = __fsub_rn(rn, rAf);
            const float F = __fmul_rn(__fmul_rn(__fmul_rn(-kf, d1), d1), __fsub_rn(rn, rSf));
            const float Fi = __fmul_rn(F, inv);
            gx = __fmaf_rn(Fi, ex, gx);
            gy = __fmaf_rn(Fi, ey, gy);
            gz = __fmaf_rn(Fi, ez, gz);
        });
        // wall: height above the surface from the bin face's height (float
        // pair) and the FP32 offset, FP64 only where no table entry exists
        float dzw;
        if (izi < G.nwz) {
            const float2 c = G.wz[izi];
            dzw = (c.x + me.z) + c.y;
        } else {
            dzw = (float)(S.z[a][i] - P.z_wall);
        }
        const float vx = gx, vy = gy, vz = gz + wall_law32(dzw, me.w, zkf, zbwf, zgf);
        const float ix = dtf * vx, iy = dtf * vy, iz = dtf * vz;
        // FP64 position accumulation
        double nx = S.x[a][i] + f2d_int(ix);
        double ny = S.y[a][i] + f2d_int(iy);
        const double nz = S.z[a][i] + f2d_int(iz);
        S.vxf[i] = vx;
        S.vyf[i] = vy;
        S.vzf[i] = vz;
        // FP32 offsets; exact FP64 re-binning near a bin face or on re-sync steps
        const float4 r = make_float4(me.x + ix, me.y + iy, me.z + iz, me.w);
        const float g0 = 1e-4f * dxb, g1 = 1e-4f * dyb, g2 = 1e-4f * dzb;
        const bool inside = !resync && r.x >= g0 && r.x <= dxb - g0 && r.y >= g1 && r.y <= dyb - g1 &&
                            r.z >= g2 && r.z <= dzb - g2;
        if (inside) {
            S.x[b][i] = nx;
            S.y[b][i] = ny;
            S.z[b][i] = nz;
            S.rel[b][i] = r;
            S.col[b][i] = col;
            S.iz[b][i] = izi;
            atomicAdd(&S.colcnt[col], 1);
            if (!isfinite(vx + vy + vz)) atomicAdd(&S.cnt->nonfinite, 1ULL);
        } else {
            if (G.per[0]) nx = wrap1(nx, G.plo[0], G.phi[0], G.len[0]);
            if (G.per[1]) ny = wrap1(ny, G.plo[1], G.phi[1], G.len[1]);
            S.x[b][i] = nx;
            S.y[b][i] = ny;
            S.z[b][i] = nz;
            rebin_slot(S, G, i, nx, ny, nz, S.rad[i], b);
        }
    }
}

}  // namespace

// k_sphere64's dynamic shared memory above the default 48 KB for 256-thread
// blocks: the attribute, once per device
template <bool SORTED>
void allow_sphere64_smem()
{
    static unsigned long long done = 0ull;  // a bit per device (set twice at worst: idempotent)
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return;
    if (dev < 64 && ((done >> dev) & 1ull)) return;
    if (cudaFuncSetAttribute(k_sphere64<SORTED>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sphere64_smem(256)) == cudaSuccess &&
        dev < 64)
        done |= 1ull << dev;
}

int launch_sphere_step(const DevState &S, const DevParams &P, double dt, int a, int precision, int grid,
                       int block, cudaStream_t st, int resync)
{
    const bool sorted = S.srel[a] != nullptr;  // the context keeps sorted copies; bare callers do not
    if (precision == BMXG_FP64_FORM) {
        // (block a multiple of 32, at most 256: the block stages and evaluates its pairs together)
        const size_t smem = sphere64_smem(block);
        if (sorted) {
            allow_sphere64_smem<true>();
            k_sphere64<true><<<grid, block, smem, st>>>(S, P, dt, a);
        } else {
            allow_sphere64_smem<false>();
            k_sphere64<false><<<grid, block, smem, st>>>(S, P, dt, a);
        }
    } else {
        if (sorted) k_sphere32<true><<<grid, block, 0, st>>>(S, P, (float)dt, a, resync);
        else k_sphere32<false><<<grid, block, 0, st>>>(S, P, (float)dt, a, resync);
    }
    return 1;
}

}  // namespace bmxg
