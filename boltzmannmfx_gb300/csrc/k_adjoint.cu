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

// ---- staged pair evaluation ----------------------------------------------
// One thread per slot walks its stencil and screens the candidates in FP32;
// the survivors (about one per slot) are staged in shared memory and the
// block then evaluates its staged pairs one per thread, so that the FP64 pair
// arithmetic runs in full warps instead of one walk iteration at a time with
// a lane or two active (GB300 issues FP64 at 2 lanes per clock per SM whatever
// the mask).  Each slot adds its pairs' terms in walk order: the same values
// in the same order as a walk that evaluates each pair when it meets it.  A
// slot with more than kStageD candidates evaluates them itself, in order.
constexpr int kStageD = 16;

// dynamic shared memory of a staged kernel: block B, NO owner values and NT
// terms per thread
__host__ __device__ constexpr size_t staged_smem(int B, int NO, int NT)
{
    return (size_t)B * (kStageD * sizeof(int2) + (NO + NT) * sizeof(double) + 4 * sizeof(int)) +
           64 * sizeof(int);
}

struct StageMem {
    int2 *stage;   // per thread: its staged candidates (j, image code)
    double *own;   // per thread: NO values of its slot for the evaluating thread
    double *term;  // per thread: NT terms of the pair it evaluated this round
    int *ocol, *orun, *olen, *opass, *wsum;
};

__device__ __forceinline__ StageMem stage_mem(unsigned char *sm, int B, int NO, int NT)
{
    StageMem M;
    M.stage = reinterpret_cast<int2 *>(sm);
    M.own = reinterpret_cast<double *>(M.stage + (size_t)B * kStageD);
    M.term = M.own + (size_t)NO * B;
    M.ocol = reinterpret_cast<int *>(M.term + (size_t)NT * B);
    M.orun = M.ocol + B;
    M.olen = M.orun + B;
    M.opass = M.olen + B;
    M.wsum = M.opass + B;
    return M;
}

// After every thread has staged its cnt candidates (and written its owner
// values and colony), the block evaluates the staged pairs one per thread:
// eval(o, e, t) computes pair e of owner thread o into t[NT] (false: no term);
// add(t) adds one term to the calling thread's sums, in staging order.
template <int NT, class Eval, class Add>
__device__ __forceinline__ void staged_pairs(const StageMem &M, int cnt, Eval &&eval, Add &&add)
{
    const int B = blockDim.x, tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = B >> 5;
    const int xl = (cnt <= kStageD) ? cnt : 0;
    int xo = xl;
    for (int d = 1; d < 32; d <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, xo, d);
        if (lane >= d) xo += v;
    }
    if (lane == 31) M.wsum[w] = xo;
    M.olen[tid] = xl;
    __syncthreads();
    if (tid == 0) {
        int run = 0;
        for (int v = 0; v < nw; ++v) {
            const int c = M.wsum[v];
            M.wsum[32 + v] = run;
            run += c;
        }
        M.wsum[31] = run;  // (at most 8 warps: slot 31 is free) the block's total
    }
    __syncthreads();
    const int xt = M.wsum[31];
    xo += M.wsum[32 + w] - xl;
    M.orun[tid] = xo;
    __syncthreads();
    for (int t0 = 0; t0 < xt; t0 += B) {
        const int t = t0 + tid;
        int pass = 0;
        double tt[NT];
        for (int c = 0; c < NT; ++c) tt[c] = 0.0;
        if (t0 + 32 * w < xt && t < xt) {  // (a warp with no pair in this round skips it)
            int o = 0;  // the slot that owns pair t: the last thread whose run starts at or before t
            for (int s2 = 1 << (31 - __clz(max(B - 1, 1))); s2 >= 1; s2 >>= 1)
                if (o + s2 < B && M.orun[o + s2] <= t) o += s2;
            pass = eval(o, M.stage[(size_t)o * kStageD + (t - M.orun[o])], tt) ? 1 : 0;
        }
        for (int c = 0; c < NT; ++c) M.term[(size_t)NT * tid + c] = tt[c];
        M.opass[tid] = pass;
        __syncthreads();
        const int k1 = min(xo + xl, t0 + B);
        for (int k = max(xo, t0); k < k1; ++k)
            if (M.opass[k - t0]) add(&M.term[(size_t)NT * (k - t0)]);
        __syncthreads();
    }
}

// The forward pair term of slot i on neighbour j (image shift sx, sy): the
// three products F u that the walk adds (false: outside the list or the cutoff).
__device__ __forceinline__ bool dfwd_term(const DevState &S, const DevGeom &G, const DevParams &P,
                                          const DiffParams &D, int a, double xi, double yi, double zi, double ri,
                                          double mi, double ai, int j, int sx, int sy, double *t)
{
    const double xj = sx ? S.x[a][j] + (double)sx * G.len[0] : S.x[a][j];
    const double yj = sy ? S.y[a][j] + (double)sy * G.len[1] : S.y[a][j];
    const double dx = xi - xj, dy = yi - yj, dz = zi - S.z[a][j];
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (!G.nbh_trivial && !(r2 <= P.nbh)) return false;
    const double rj = S.rad[j];
    const double rlm = ri + rj + P.bw;
    if (!(r2 <= (rlm - kSmall) * (rlm - kSmall))) return false;
    const double rS = ri + rj, rA = rS + P.bw;
    const double rn = sqrt(r2);
    const double ux = dx / rn, uy = dy / rn, uz = dz / rn;
    const double abar = 0.5 * (ai + (D.adh ? D.adh[j] : 0.0));
    const PairLaw q = pair_law(rn, rS, rA, P.k, P.bw, abar);
    const double s = 1.0 / (1.0 + D.gamma * (mi + mobility_of(rj, D.mu)));
    const double F = mi * (q.f * s);
    t[0] = F * ux;
    t[1] = F * uy;
    t[2] = F * uz;
    return true;
}

// The adjoint pair term of slot k on neighbour j: its contribution to the
// gathered J w (t[0..2]) and to the stiffness, damping, drag and adhesion
// slopes (t[3..6]) (false: no contribution).
__device__ __forceinline__ bool dadj_term(const DevState &S, const DevGeom &G, const DevParams &P,
                                          const DiffParams &D, int a, const double *__restrict__ lin, int n,
                                          const double *o, int j, int sx, int sy, double *t)
{
    // o: xk, yk, zk, rk, mk, dmk, ak, lk[3]
    const double xk = o[0], yk = o[1], zk = o[2], rk = o[3], mk = o[4], dmk = o[5], ak = o[6];
    const double lk[3] = {o[7], o[8], o[9]};
    const double xj = sx ? S.x[a][j] + (double)sx * G.len[0] : S.x[a][j];
    const double yj = sy ? S.y[a][j] + (double)sy * G.len[1] : S.y[a][j];
    const double d[3] = {xk - xj, yk - yj, zk - S.z[a][j]};
    const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    if (!G.nbh_trivial && !(r2 <= P.nbh)) return false;
    const double rj = S.rad[j];
    const double rlm = rk + rj + P.bw;
    if (!(r2 <= (rlm - kSmall) * (rlm - kSmall))) return false;
    const double rS = rk + rj, rA = rS + P.bw;
    const double rn = sqrt(r2);
    if (!(rn < rA)) return false;  // f, f' and all parameter slopes vanish
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
    for (int c = 0; c < 3; ++c) t[c] = dFt * u[c] * uw + fr * (w[c] - u[c] * uw);
    // parameter slopes of v_k (this pair's term m_k Ft u), against lam'_k
    const double lu = lk[0] * u[0] + lk[1] * u[1] + lk[2] * u[2];
    t[3] = mk * (q.fk * s) * lu;
    t[4] = mk * (-q.f * M * s * s) * lu;
    t[5] = (dmk * Ft + mk * (-q.f * s * s * D.gamma * (dmk + dmj))) * lu;
    // adhesion of k enters both v_k and v_j through abar = (a_k + a_j)/2
    t[6] = 0.5 * (q.fa * s) * uw;
    return true;
}

// forward step of the differentiable form (reads buffer a, writes b, rebins)
template <bool SORTED>
__global__ void __launch_bounds__(256) k_dfwd(const DevState S, const DevParams P, DiffParams D, double dt, int a)
{
    extern __shared__ __align__(16) unsigned char smd[];
    constexpr int NO = 6, NT = 3;
    const int B = blockDim.x, tid = threadIdx.x;
    const StageMem M = stage_mem(smd, B, NO, NT);
    const int b = a ^ 1;
    const float bwf = P.bw32;
    for (int base = blockIdx.x * B; base < S.n; base += gridDim.x * B) {
        const int i = base + tid;
        const bool act = i < S.n;
        double xi = 0.0, yi = 0.0, zi = 0.0, ri = 0.0, mi = 0.0, ai = 0.0;
        double fx = 0.0, fy = 0.0, fz = 0.0;
        int col = 0, cnt = 0;
        if (act) {
            col = colony_of(S.cbase, S.ncol, i);
            const DevGeom &G = S.geoms[col];
            int bx, by;
            col_to_bxy(G, S.col[a][i], bx, by);
            xi = S.x[a][i];
            yi = S.y[a][i];
            zi = S.z[a][i];
            ri = S.rad[i];
            mi = mobility_of(ri, D.mu);
            ai = D.adh ? D.adh[i] : 0.0;
            const float4 me = S.rel[a][i];
            const float slack = screen_slack(G);
            int2 *mine = M.stage + (size_t)tid * kStageD;
            auto eval = [&](int j, int sx, int sy) {
                double t[3];
                if (dfwd_term(S, G, P, D, a, xi, yi, zi, ri, mi, ai, j, sx, sy, t)) {
                    fx += t[0];
                    fy += t[1];
                    fz += t[2];
                }
            };
            walk<SORTED>(S, G, a, i, bx, by, S.iz[a][i], [&](const float4 qr, auto slot, int dxs, int dys, int dzs,
                                                             int sx, int sy) {
                if (!near32(me, qr, dxs, dys, dzs, G, bwf, slack)) return;
                const int j = slot();
                if (cnt < kStageD) {
                    mine[cnt] = make_int2(j, (sx + 1) * 3 + (sy + 1));
                } else {
                    if (cnt == kStageD)  // too many for the stage: the staged ones first, in order
                        for (int k = 0; k < kStageD; ++k) eval(mine[k].x, mine[k].y / 3 - 1, mine[k].y % 3 - 1);
                    eval(j, sx, sy);
                }
                ++cnt;
            });
        }
        double *own = M.own + (size_t)NO * tid;
        own[0] = xi;
        own[1] = yi;
        own[2] = zi;
        own[3] = ri;
        own[4] = mi;
        own[5] = ai;
        M.ocol[tid] = col;
        staged_pairs<NT>(
            M, cnt,
            [&](int o, int2 e, double *t) {
                const double *oo = M.own + (size_t)NO * o;
                return dfwd_term(S, S.geoms[M.ocol[o]], P, D, a, oo[0], oo[1], oo[2], oo[3], oo[4], oo[5], e.x,
                                 e.y / 3 - 1, e.y % 3 - 1, t);
            },
            [&](const double *t) {
                fx += t[0];
                fy += t[1];
                fz += t[2];
            });
        if (act) {
            const DevGeom &G = S.geoms[col];
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
        __syncthreads();  // the next pass reuses the stage and the slot records
    }
}

// adjoint of the step taken from buffer a (positions x_t, bins of x_t)
template <bool SORTED>
__global__ void __launch_bounds__(256) k_dadj(const DevState S, const DevParams P, DiffParams D, double dt, int a,
                                             const double *__restrict__ lin, double *__restrict__ lout,
                                             double *__restrict__ gacc, double *__restrict__ gadh)
{
    extern __shared__ __align__(16) unsigned char smd[];
    constexpr int NO = 10, NT = 7;
    const int B = blockDim.x, tid = threadIdx.x;
    const StageMem M = stage_mem(smd, B, NO, NT);
    const int n = S.n;
    const float bwf = P.bw32;
    for (int base = blockIdx.x * B; base < n; base += gridDim.x * B) {
        const int k = base + tid;
        const bool act = k < n;
        double o[NO];
        for (int c = 0; c < NO; ++c) o[c] = 0.0;
        double acc[3] = {0.0, 0.0, 0.0};
        double gk = 0.0, gg = 0.0, gm = 0.0, ga = 0.0;
        int col = 0, cnt = 0;
        auto add = [&](const double *t) {
            for (int c = 0; c < 3; ++c) acc[c] += t[c];
            gk += t[3];
            gg += t[4];
            gm += t[5];
            ga += t[6];
        };
        if (act) {
            col = colony_of(S.cbase, S.ncol, k);
            const DevGeom &G = S.geoms[col];
            int bx, by;
            col_to_bxy(G, S.col[a][k], bx, by);
            const double rk = S.rad[k];
            const double mk = mobility_of(rk, D.mu);
            o[0] = S.x[a][k];
            o[1] = S.y[a][k];
            o[2] = S.z[a][k];
            o[3] = rk;
            o[4] = mk;
            o[5] = D.mu > 0.0 ? -mk / D.mu : 0.0;
            o[6] = D.adh ? D.adh[k] : 0.0;
            o[7] = lin[k];
            o[8] = lin[(size_t)n + k];
            o[9] = lin[(size_t)2 * n + k];
            const float4 me = S.rel[a][k];
            const float slack = screen_slack(G);
            int2 *mine = M.stage + (size_t)tid * kStageD;
            auto eval = [&](int j, int sx, int sy) {
                double t[NT];
                if (dadj_term(S, G, P, D, a, lin, n, o, j, sx, sy, t)) add(t);
            };
            walk<SORTED>(S, G, a, k, bx, by, S.iz[a][k], [&](const float4 qr, auto slot, int dxs, int dys, int dzs,
                                                             int sx, int sy) {
                if (!near32(me, qr, dxs, dys, dzs, G, bwf, slack)) return;
                const int j = slot();
                if (cnt < kStageD) {
                    mine[cnt] = make_int2(j, (sx + 1) * 3 + (sy + 1));
                } else {
                    if (cnt == kStageD)
                        for (int q = 0; q < kStageD; ++q) eval(mine[q].x, mine[q].y / 3 - 1, mine[q].y % 3 - 1);
                    eval(j, sx, sy);
                }
                ++cnt;
            });
        }
        for (int c = 0; c < NO; ++c) M.own[(size_t)NO * tid + c] = o[c];
        M.ocol[tid] = col;
        staged_pairs<NT>(
            M, cnt,
            [&](int ow, int2 e, double *t) {
                return dadj_term(S, S.geoms[M.ocol[ow]], P, D, a, lin, n, M.own + (size_t)NO * ow, e.x,
                                 e.y / 3 - 1, e.y % 3 - 1, t);
            },
            add);
        if (act) {
            const double wz = wall_slope(o[2], o[3], P);
            lout[k] = o[7] + dt * acc[0];
            lout[(size_t)n + k] = o[8] + dt * acc[1];
            lout[(size_t)2 * n + k] = o[9] + dt * (acc[2] + wz * o[9]);
            gacc[k] += dt * gk;
            gacc[(size_t)n + k] += dt * gg;
            gacc[(size_t)2 * n + k] += dt * gm;
            gadh[k] += dt * ga;
        }
        __syncthreads();
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

// a kernel's dynamic shared memory above the default 48 KB (the launches
// that need it: 256-thread blocks)
template <class K>
void allow_smem(K kernel, size_t need)
{
    if (need > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need);
}

int launch_dfwd(const DevState &S, const DevParams &P, const DiffParams &D, double dt, int a, int grid, int block,
                cudaStream_t st)
{
    const size_t smem = staged_smem(block, 6, 3);
    if (S.srel[a]) {
        allow_smem(k_dfwd<true>, smem);
        k_dfwd<true><<<grid, block, smem, st>>>(S, P, D, dt, a);
    } else {
        allow_smem(k_dfwd<false>, smem);
        k_dfwd<false><<<grid, block, smem, st>>>(S, P, D, dt, a);
    }
    return 1;
}

int launch_dadj(const DevState &S, const DevParams &P, const DiffParams &D, double dt, int a, const double *lin,
                double *lout, double *gacc, double *gadh, int grid, int block, cudaStream_t st)
{
    const size_t smem = staged_smem(block, 10, 7);
    if (S.srel[a]) {
        allow_smem(k_dadj<true>, smem);
        k_dadj<true><<<grid, block, smem, st>>>(S, P, D, dt, a, lin, lout, gacc, gadh);
    } else {
        allow_smem(k_dadj<false>, smem);
        k_dadj<false><<<grid, block, smem, st>>>(S, P, D, dt, a, lin, lout, gacc, gadh);
    }
    return 1;
}

int launch_dreduce(const double *gacc, int n, int planes, double *out, cudaStream_t st)
{
    k_dreduce<<<1, 256, 0, st>>>(gacc, n, planes, out);
    return 1;
}

}  // namespace bmxg
