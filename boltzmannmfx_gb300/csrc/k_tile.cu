// k_tile.cu -- the FP64 sphere step of one tile with the caller's ghost
// particles: AMReX's per-tile EvolveParticles (src/des/bmx_pc_interaction.cpp:
// 97-279 with the halo of one cell of src/des/bmx_pc.cpp:23), where
// fillNeighbors has put copies of the particles of the neighbouring tiles --
// periodic images already shifted by a domain length -- beside the tile's own.
//
// The tile's cells are the level's global cells (the particle's cell from the
// domain origin, as the whole-domain step bins it) offset by the tile's first
// cell; the grown box adds the one-cell halo that holds the ghosts.  A real
// particle walks the 27 cells around its own in the whole-domain step's
// order (x outermost, then y, then z, ascending index within a cell: the
// tile's reals in the caller's order, then its ghosts in theirs), and each
// pair is evaluated with the whole-domain step's FP64 operations on the
// ghost's given position.  So with the ghosts a whole-domain step would see
// (copies of every particle within one cell of the tile, images at x + s L),
// the tiles' results are bit-identical to the step of the whole domain.
#include <algorithm>

#include "bmxg_stencil.cuh"

namespace bmxg {

namespace {

__device__ __forceinline__ int tile_cell(const TileGeom &T, int lx, int ly, int lz)
{
    return (lx * (T.nt[1] + 2) + ly) * (T.nt[2] + 2) + lz;
}

// Cell of every particle (reals [0, nreal), then ghosts) in the grown tile
// box and the per-cell counts.  bad[0] counts a real outside the tile or a
// ghost outside the halo, bad[1] a particle that is not a sphere (YEAST).
__global__ void k_tile_bin(const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
                           const int *__restrict__ ct, int nreal, int ntot, TileGeom T, int *cell, int *cnt,
                           unsigned long long *bad)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < ntot; p += gridDim.x * blockDim.x) {
        const double pos[3] = {x[p], y[p], z[p]};
        const bool real = p < nreal;
        int l[3];
        bool halo = false, out = false;
        for (int d = 0; d < 3; ++d) {
            // the whole-domain step's bin (1-based): a slot's own clamped to the
            // domain, a periodic image's the halo cell its shifted position is in
            const int gb = (real || !T.per[d]) ? bin_of(pos[d], T.plo[d], T.dxi[d], 1, T.n[d])
                                                : bin_of(pos[d], T.plo[d], T.dxi[d], 0, T.n[d] + 1);
            int lb = gb - T.lo[d];
            if (lb < 0 || lb > T.nt[d] + 1) {
                out = true;
                lb = min(max(lb, 0), T.nt[d] + 1);
            }
            if (lb == 0 || lb == T.nt[d] + 1) halo = true;
            l[d] = lb;
        }
        if (out || (real ? halo : !halo)) atomicAdd(&bad[0], 1ull);
        if (ct[p] != kYeast) atomicAdd(&bad[1], 1ull);
        const int c = tile_cell(T, l[0], l[1], l[2]);
        cell[p] = c;
        atomicAdd(&cnt[c], 1);
    }
}

__global__ void k_tile_scatter(const int *__restrict__ cell, int ntot, const int *__restrict__ start, int *fill,
                               int *perm)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < ntot; p += gridDim.x * blockDim.x) {
        const int c = cell[p];
        perm[start[c] + atomicAdd(&fill[c], 1)] = p;
    }
}

// ascending index within each cell (the scatter's arrival order is arbitrary)
__global__ void k_tile_order(const int *__restrict__ start, int ncells, int *perm)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += gridDim.x * blockDim.x) {
        const int lo = start[c], hi = start[c + 1];
        for (int t = lo + 1; t < hi; ++t) {
            const int v = perm[t];
            int u = t - 1;
            while (u >= lo && perm[u] > v) {
                perm[u + 1] = perm[u];
                --u;
            }
            perm[u + 1] = v;
        }
    }
}

__global__ void __launch_bounds__(128) k_tile_step(const double *__restrict__ x, const double *__restrict__ y,
                                                   const double *__restrict__ z, const double *__restrict__ r,
                                                   int nreal, const int *__restrict__ cell,
                                                   const int *__restrict__ start, const int *__restrict__ perm,
                                                   TileGeom T, DevParams P, double dt, double *ox, double *oy,
                                                   double *oz, double *vx, double *vy, double *vz,
                                                   unsigned long long *bad)
{
    const int nz2 = T.nt[2] + 2, nyz = (T.nt[1] + 2) * nz2;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nreal; i += gridDim.x * blockDim.x) {
        const int c = cell[i];
        const int lx = c / nyz, ly = (c / nz2) % (T.nt[1] + 2), lz = c % nz2;
        const double xi = x[i], yi = y[i], zi = z[i], ri = r[i];
        double fx = 0.0, fy = 0.0, fz = 0.0;
        for (int dxs = -1; dxs <= 1; ++dxs) {
            for (int dys = -1; dys <= 1; ++dys) {
                for (int dzs = -1; dzs <= 1; ++dzs) {
                    // (a real outside its tile, an input error the call reports,
                    // has cells outside the grown box: skipped)
                    if (lx + dxs < 0 || lx + dxs > T.nt[0] + 1 || ly + dys < 0 || ly + dys > T.nt[1] + 1 ||
                        lz + dzs < 0 || lz + dzs > T.nt[2] + 1)
                        continue;
                    const int cc = tile_cell(T, lx + dxs, ly + dys, lz + dzs);
                    const int hi = start[cc + 1];
                    for (int t = start[cc]; t < hi; ++t) {
                        const int j = perm[t];
                        if (j == i) continue;
                        // the whole-domain step's pair term (k_sphere64), on the
                        // ghost's given position
                        const double dx = xi - x[j], dy = yi - y[j], dz = zi - z[j];
                        const double r2 = dx * dx + dy * dy + dz * dz;
                        if (!T.nbh_trivial && !(r2 <= P.nbh)) continue;  // not in the neighbour list
                        const double rj = r[j];
                        const double rlm = ri + rj + P.bw;                // maxInteractionDistance
                        if (!(r2 <= (rlm - kSmall) * (rlm - kSmall))) continue;
                        const double rS = ri + rj;
                        const double rA = rS + P.bw;
                        const double rn = sqrt(r2);
                        const double ux = dx / rn, uy = dy / rn, uz = dz / rn;
                        const double F = (rn < rA) ? -P.k * (rn - rA) * (rn - rA) * (rn - rS) : 0.0;
                        fx += F * ux;
                        fy += F * uy;
                        fz += F * uz;
                    }
                }
            }
        }
        // evaluateSurfaceForce (sphere branch), the update, and the periodic
        // wrap of the trailing Redistribute, as the whole-domain step
        const double v0 = fx + 0.0;
        const double v1 = fy + 0.0;
        const double v2 = fz + wall_law(zi, ri, P);
        double nx = xi + dt * v0;
        double ny = yi + dt * v1;
        const double nz = zi + dt * v2;
        if (T.per[0]) nx = wrap1(nx, T.plo[0], T.phi[0], T.len[0]);
        if (T.per[1]) ny = wrap1(ny, T.plo[1], T.phi[1], T.len[1]);
        if (!finite_bits(nx) || !finite_bits(ny) || !finite_bits(nz)) atomicAdd(&bad[2], 1ull);
        ox[i] = nx;
        oy[i] = ny;
        oz[i] = nz;
        vx[i] = v0;
        vy[i] = v1;
        vz[i] = v2;
    }
}

}  // namespace

int launch_tile_step(const TileBufs &B, const TileGeom &T, const DevParams &P, double dt, int nreal, int ntot,
                     int *scan_scratch, int nsm, cudaStream_t st)
{
    const int ncells = (T.nt[0] + 2) * (T.nt[1] + 2) * (T.nt[2] + 2);
    const int blk = 256;
    const int gp = std::max(1, std::min((ntot + blk - 1) / blk, nsm * 8));
    const int gc = std::max(1, std::min((ncells + blk - 1) / blk, nsm * 8));
    k_tile_bin<<<gp, blk, 0, st>>>(B.x, B.y, B.z, B.ct, nreal, ntot, T, B.cell, B.cnt, B.bad);
    int k = 1 + launch_scan(B.cnt, B.start, ncells, scan_scratch, st, nullptr);
    k_tile_scatter<<<gp, blk, 0, st>>>(B.cell, ntot, B.start, B.fill, B.perm);
    k_tile_order<<<gc, blk, 0, st>>>(B.start, ncells, B.perm);
    k_tile_step<<<std::max(1, std::min((nreal + 127) / 128, nsm * 16)), 128, 0, st>>>(
        B.x, B.y, B.z, B.r, nreal, B.cell, B.start, B.perm, T, P, dt, B.ox, B.oy, B.oz, B.vx, B.vy, B.vz, B.bad);
    return k + 3;
}

}  // namespace bmxg
