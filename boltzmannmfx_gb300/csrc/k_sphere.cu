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
//  FP64  (plain)  every pair that can pass the reference's cutoff test is
//                 evaluated in FP64 with the reference's operation order
//                 (this file is compiled with -fmad=false), accumulated in
//                 list order: the result is bit-identical to the host
//                 oracle.  Pairs are first screened in FP32 from the
//                 bin-relative offsets with an absolute slack that bounds the
//                 FP32 error, so only pairs that are certainly beyond the
//                 cutoff skip the FP64 test.
//  FP32F (precision form) pair math in FP32 on FP64-differenced bin-relative
//                 offsets; the wall force and the position accumulation stay
//                 FP64.
// Roofline: HBM / L2 bound gather; no dense contraction, so no tensor cores.
#include "bmxg_stencil.cuh"

namespace bmxg {

namespace {

template <int PREC>
__global__ void __launch_bounds__(256) k_sphere(const DevState S, const DevParams P, double dt, int a)
{
    const int b = a ^ 1;
    const float bwf = (float)P.bw;
    const float kf = (float)P.k;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += gridDim.x * blockDim.x) {
        const DevGeom &G = geom_of(S, i);
        int bx, by;
        col_to_bxy(G, S.col[a][i], bx, by);
        const int izi = S.iz[a][i];
        const double xi = S.x[a][i], yi = S.y[a][i], zi = S.z[a][i];
        const double ri = S.rad[i];
        const float4 me = S.rel[a][i];
        const float dxb = G.dxf[0], dyb = G.dxf[1], dzb = G.dxf[2];
        // absolute slack bounding the FP32 distance error (offsets + bin widths)
        const float slack = 8.0f * 1.1920929e-7f * fmaxf(dxb, fmaxf(dyb, dzb));
        double fx = 0.0, fy = 0.0, fz = 0.0;
        float gx = 0.0f, gy = 0.0f, gz = 0.0f;
        visit_stencil(S, G, a, i, bx, by, izi, [&](int j, int dxs, int dys, int dzs, int sx, int sy) {
            const float4 q = __ldg(&S.rel[a][j]);
            const float ex = (me.x - q.x) - (float)dxs * dxb;
            const float ey = (me.y - q.y) - (float)dys * dyb;
            const float ez = (me.z - q.z) - (float)dzs * dzb;
            const float r2f = __fmaf_rn(ex, ex, __fmaf_rn(ey, ey, __fmul_rn(ez, ez)));
            const float rAf = __fadd_rn(__fadd_rn(me.w, q.w), bwf);
            if (PREC == BMXG_FP64_FORM) {
                const float lim = __fadd_rn(rAf, slack);
                if (r2f > __fmul_rn(lim, lim)) return;
                const double xj = sx ? S.x[a][j] + (double)sx * G.len[0] : S.x[a][j];
                const double yj = sy ? S.y[a][j] + (double)sy * G.len[1] : S.y[a][j];
                const double dx = xi - xj, dy = yi - yj, dz = zi - S.z[a][j];
                const double r2 = dx * dx + dy * dy + dz * dz;
                if (!G.nbh_trivial && !(r2 <= P.nbh)) return;  // not in the neighbour list
                const double rj = S.rad[j];
                const double rlm = ri + rj + P.bw;                // maxInteractionDistance
                if (!(r2 <= (rlm - kSmall) * (rlm - kSmall))) return;
                const double rS = ri + rj;
                const double rA = rS + P.bw;
                const double rn = sqrt(r2);
                const double ux = dx / rn, uy = dy / rn, uz = dz / rn;
                const double F = (rn < rA) ? -P.k * (rn - rA) * (rn - rA) * (rn - rS) : 0.0;
                fx += F * ux;
                fy += F * uy;
                fz += F * uz;
            } else {
                if (!(r2f < __fmul_rn(rAf, rAf))) return;
                if (!G.nbh_trivial) {
                    const double xj = sx ? S.x[a][j] + (double)sx * G.len[0] : S.x[a][j];
                    const double yj = sy ? S.y[a][j] + (double)sy * G.len[1] : S.y[a][j];
                    const double dx = xi - xj, dy = yi - yj, dz = zi - S.z[a][j];
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
            }
        });
        if (PREC != BMXG_FP64_FORM) {
            fx = (double)gx;
            fy = (double)gy;
            fz = (double)gz;
        }
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
}

}  // namespace

int launch_sphere_step(const DevState &S, const DevParams &P, double dt, int a, int precision, int grid,
                        int block, cudaStream_t st)
{
    if (precision == BMXG_FP64_FORM)
        k_sphere<BMXG_FP64_FORM><<<grid, block, 0, st>>>(S, P, dt, a);
    else
        k_sphere<BMXG_FP32F_FORM><<<grid, block, 0, st>>>(S, P, dt, a);
    return 1;
}

}  // namespace bmxg
