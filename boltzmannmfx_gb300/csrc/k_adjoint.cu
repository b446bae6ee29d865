// k_adjoint.cu -- the differentiation form: an FP64 sphere step with the
// contact-parameter extensions, and its hand-written adjoint.
//
// Forward law (spheres; the reference law of
// src/chemistry/bmx_cell_interaction_K.H:243-276 and :1009-1030 when
// damping = mu = adhesion = 0, bit for bit):
//   f(r)   = -k (r - rA)^2 (r - rS) - k bw abar (r - rA)^2        r < rA
//   Ft(r)  = f(r) / (1 + gamma (m_i + m_j))      two-body overdamped dashpot
//   v_i    = m_i sum_j Ft(r_ij) u_ij + wall(z_i) e_z
//   x_i'   = x_i + dt v_i                        (then the periodic wrap)
// with abar = (a_i + a_j)/2 (per-particle adhesion energy, in units of the
// band's spring energy), m_i = 1/(6 pi mu r_i) for mu > 0 and 1 otherwise
// (drag folded into k, as the reference does).
//
// Adjoint of one step, lam' = dL/dx_{t+1}:
//   lam_k = lam'_k + dt [ sum_j J_kj (m_k lam'_k - m_j lam'_j) + wall'(z_k) lam'_kz e_z ]
//   J = Ft' u u^T + (Ft / r)(I - u u^T)   (symmetric, J_kj = J_jk)
// a gather over the same neighbour walk as the forward step -- no atomics.
// Parameter gradients are accumulated per slot across steps (deterministic)
// and reduced once at the end.
#include "bmxg_stencil.cuh"

namespace bmxg {

namespace {

struct PairLaw {
    double f, df, fk, fa;  // f, df/dr, df/dk, df/dabar
};

__device__ __forceinline__ PairLaw pair_law(double r, double rS, double rA, double k, double bw, double abar)
{
    PairLaw q{0.0, 0.0, 0.0, 0.0};
    if (r < rA) {
        const double e = r - rA, g = r - rS;
        q.f = -k * e * e * g - k * bw * abar * e * e;
        q.df = -k * (2.0 * e * g + e * e) - 2.0 * k * bw * abar * e;
        q.fk = -e * e * g - bw * abar * e * e;
        q.fa = -k * bw * e * e;
    }
    return q;
}

__device__ __forceinline__ double mobility_of(double r, double mu)
{
    return mu > 0.0 ? 1.0 / (6.0 * kPi * mu * r) : 1.0;
}

__device__ __forceinline__ double wall_slope(double z, double rS, const DevParams &P)
{
    const double dz = z - P.z_wall;
    const double rA = rS + P.z_bw;
    if (dz > 0.0 && dz < rA) return -P.z_k * (2.0 * (dz - rA) * (dz - rS) + (dz - rA) * (dz - rA));
    return 0.0;
}

// The FP32 screen of the FP64 pair walks (as in the FP64 sphere step): false
// only when the candidate is certainly beyond the cutoff r_i + r_j + bw, from
// the FP32 offsets to the bin corners with an absolute slack of 8 ulp of the
// largest bin width that bounds their error; the FP64 gate decides the rest.
__device__ __forceinline__ bool near32(const float4 me, const float4 q, int dxs, int dys, int dzs, const DevGeom &G,
                                       float bwf, float slack)
{
    const float ex = (me.x - q.x) - (float)dxs * G.dxf[0];
    const float ey = (me.y - q.y) - (float)dys * G.dxf[1];
    const float ez = (me.z - q.z) - (float)dzs * G.dxf[2];
    const float r2f = __fmaf_rn(ex, ex, __fmaf_rn(ey, ey, __fmul_rn(ez, ez)));
    const float lim = __fadd_rn(__fadd_rn(__fadd_rn(me.w, q.w), bwf), slack);
    return !(r2f > __fmul_rn(lim, lim));
}

__device__ __forceinline__ float screen_slack(const DevGeom &G)
{
    return 8.0f * 1.1920929e-7f * fmaxf(G.dxf[0], fmaxf(G.dxf[1], G.dxf[2]));
}

// forward step of the differentiable form (reads buffer a, writes b, rebins)
template <bool SORTED>
__global__ void __launch_bounds__(256) k_dfwd(const DevState S, const DevParams P, DiffParams D, double dt, int a)
{
    const int b = a ^ 1;
    const float bwf = P.bw32;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += gridDim.x * blockDim.x) {
        const DevGeom &G = geom_of(S, i);
        int bx, by;
        col_to_bxy(G, S.col[a][i], bx, by);
        const double xi = S.x[a][i], yi = S.y[a][i], zi = S.z[a][i];
        const double ri = S.rad[i];
        const double mi = mobility_of(ri, D.mu);
        const double ai = D.adh ? D.adh[i] : 0.0;
        const float4 me = S.rel[a][i];
        const float slack = screen_slack(G);
        double fx = 0.0, fy = 0.0, fz = 0.0;
        walk<SORTED>(S, G, a, i, bx, by, S.iz[a][i], [&](const float4 qr, auto slot, int dxs, int dys, int dzs,
                                                         int sx, int sy) {
            if (!near32(me, qr, dxs, dys, dzs, G, bwf, slack)) return;
            const int j = slot();
            const double xj = sx ? S.x[a][j] + (double)sx * G.len[0] : S.x[a][j];
            const double yj = sy ? S.y[a][j] + (double)sy * G.len[1] : S.y[a][j];
            const double dx = xi - xj, dy = yi - yj, dz = zi - S.z[a][j];
            const double r2 = dx * dx + dy * dy + dz * dz;
            if (!G.nbh_trivial && !(r2 <= P.nbh)) return;
            const double rj = S.rad[j];
            const double rlm = ri + rj + P.bw;
            if (!(r2 <= (rlm - kSmall) * (rlm - kSmall))) return;
            const double rS = ri + rj, rA = rS + P.bw;
            const double rn = sqrt(r2);
            const double ux = dx / rn, uy = dy / rn, uz = dz / rn;
            const double abar = 0.5 * (ai + (D.adh ? D.adh[j] : 0.0));
            const PairLaw q = pair_law(rn, rS, rA, P.k, P.bw, abar);
            const double s = 1.0 / (1.0 + D.gamma * (mi + mobility_of(rj, D.mu)));
            const double F = mi * (q.f * s);
            fx += F * ux;
            fy += F * uy;
            fz += F * uz;
        });
        const double vx = fx + 0.0, vy = fy + 0.0, vz = fz + wall_law(zi, ri, P);
        double nx = xi + dt * vx, ny = yi + dt * vy;
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

// adjoint of the step taken from buffer a (positions x_t, bins of x_t)
template <bool SORTED>
__global__ void __launch_bounds__(256) k_dadj(const DevState S, const DevParams P, DiffParams D, double dt, int a,
                                             const double *__restrict__ lin, double *__restrict__ lout,
                                             double *__restrict__ gacc, double *__restrict__ gadh)
{
    const int n = S.n;
    const float bwf = P.bw32;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const DevGeom &G = geom_of(S, k);
        int bx, by;
        col_to_bxy(G, S.col[a][k], bx, by);
        const double xk = S.x[a][k], yk = S.y[a][k], zk = S.z[a][k];
        const double rk = S.rad[k];
        const double mk = mobility_of(rk, D.mu);
        const double dmk = D.mu > 0.0 ? -mk / D.mu : 0.0;
        const double ak = D.adh ? D.adh[k] : 0.0;
        const double lk[3] = {lin[k], lin[(size_t)n + k], lin[(size_t)2 * n + k]};
        double acc[3] = {0.0, 0.0, 0.0};
        double gk = 0.0, gg = 0.0, gm = 0.0, ga = 0.0;
        const float4 me = S.rel[a][k];
        const float slack = screen_slack(G);
        walk<SORTED>(S, G, a, k, bx, by, S.iz[a][k], [&](const float4 qr, auto slot, int dxs, int dys, int dzs,
                                                         int sx, int sy) {
            if (!near32(me, qr, dxs, dys, dzs, G, bwf, slack)) return;
            const int j = slot();
            const double xj = sx ? S.x[a][j] + (double)sx * G.len[0] : S.x[a][j];
            const double yj = sy ? S.y[a][j] + (double)sy * G.len[1] : S.y[a][j];
            const double d[3] = {xk - xj, yk - yj, zk - S.z[a][j]};
            const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (!G.nbh_trivial && !(r2 <= P.nbh)) return;
            const double rj = S.rad[j];
            const double rlm = rk + rj + P.bw;
            if (!(r2 <= (rlm - kSmall) * (rlm - kSmall))) return;
            const double rS = rk + rj, rA = rS + P.bw;
            const double rn = sqrt(r2);
            if (!(rn < rA)) return;  // f, f' and all parameter slopes vanish
            const double u[3] = {d[0] / rn, d[1] / rn, d[2] / rn};
            const double mj = mobility_of(rj, D.mu);
            const double dmj = D.mu > 0.0 ? -mj / D.mu : 0.0;
            const double abar = 0.5 * (ak + (D.adh ? D.adh[j] : 0.0));
            const PairLaw q = pair_law(rn, rS, rA, P.k, P.bw, abar);
            const double M = mk + mj;
            const double s = 1.0 / (1.0 + D.gamma * M);
            const double Ft = q.f * s, dFt = q.df * s;
            const double lj[3] = {lin[j], lin[(size_t)n + j], lin[(size_t)2 * n + j]};
            // w = m_k lam'_k - m_j lam'_j ; J w = dFt u (u.w) + (Ft/r)(w - u (u.w))
            double w[3];
            for (int c = 0; c < 3; ++c) w[c] = mk * lk[c] - mj * lj[c];
            const double uw = u[0] * w[0] + u[1] * w[1] + u[2] * w[2];
            const double fr = Ft / rn;
            for (int c = 0; c < 3; ++c) acc[c] += dFt * u[c] * uw + fr * (w[c] - u[c] * uw);
            // parameter slopes of v_k (this pair's term m_k Ft u), against lam'_k
            const double lu = lk[0] * u[0] + lk[1] * u[1] + lk[2] * u[2];
            gk += mk * (q.fk * s) * lu;
            gg += mk * (-q.f * M * s * s) * lu;
            gm += (dmk * Ft + mk * (-q.f * s * s * D.gamma * (dmk + dmj))) * lu;
            // adhesion of k enters both v_k and v_j through abar = (a_k + a_j)/2
            ga += 0.5 * (q.fa * s) * uw;
        });
        const double wz = wall_slope(zk, rk, P);
        lout[k] = lk[0] + dt * acc[0];
        lout[(size_t)n + k] = lk[1] + dt * acc[1];
        lout[(size_t)2 * n + k] = lk[2] + dt * (acc[2] + wz * lk[2]);
        gacc[k] += dt * gk;
        gacc[(size_t)n + k] += dt * gg;
        gacc[(size_t)2 * n + k] += dt * gm;
        gadh[k] += dt * ga;
    }
}

// deterministic sum of per-slot gradient planes (one block, fixed order)
__global__ void k_dreduce(const double *gacc, int n, int planes, double *out)
{
    __shared__ double sh[256];
    for (int p = 0; p < planes; ++p) {
        double s = 0.0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) s += gacc[(size_t)p * n + i];
        sh[threadIdx.x] = s;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[p] = sh[0];
        __syncthreads();
    }
}

}  // namespace

int launch_dfwd(const DevState &S, const DevParams &P, const DiffParams &D, double dt, int a, int grid, int block,
                cudaStream_t st)
{
    if (S.srel[a]) k_dfwd<true><<<grid, block, 0, st>>>(S, P, D, dt, a);
    else k_dfwd<false><<<grid, block, 0, st>>>(S, P, D, dt, a);
    return 1;
}

int launch_dadj(const DevState &S, const DevParams &P, const DiffParams &D, double dt, int a, const double *lin,
                double *lout, double *gacc, double *gadh, int grid, int block, cudaStream_t st)
{
    if (S.srel[a]) k_dadj<true><<<grid, block, 0, st>>>(S, P, D, dt, a, lin, lout, gacc, gadh);
    else k_dadj<false><<<grid, block, 0, st>>>(S, P, D, dt, a, lin, lout, gacc, gadh);
    return 1;
}

int launch_dreduce(const double *gacc, int n, int planes, double *out, cudaStream_t st)
{
    k_dreduce<<<1, 256, 0, st>>>(gacc, n, planes, out);
    return 1;
}

}  // namespace bmxg
