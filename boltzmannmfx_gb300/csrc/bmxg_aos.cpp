// bmxg_aos.cpp -- the step on particles stored in the reference's own layout.
//
// BMX keeps its particles as amrex::Particle<MAX_CHEM_REAL_VAR = 34,
// MAX_CHEM_INT_VAR = 35> (src/chemistry/bmx_chem.H:16-17, container
// src/des/bmx_pc.H:86-100): in AMReX 22.x with double precision that is
//   double pos[3]; double rdata[nreal]; int id; int cpu; int idata[nint];
// padded to 8 bytes (448 bytes for 34 / 35).  bmxg_evolve_particles_aos takes
// a host array of such structs (one tile's ParticleTile::GetArrayOfStructs()
// data), runs one DEM step through the SoA entry points and writes back what
// the reference's step writes: pos, velx..velz, wx..wz, theta, phi and the
// integer fields its pair loop and wall force touch.
#include <cstddef>
#include <cstring>
#include <vector>

#include "../../include/bmxg.h"

namespace {

// realIdx (src/chemistry/bmx_chem.H:38-69)
enum {
    R_radius = 0, R_c_length = 1, R_theta = 2, R_phi = 3, R_area = 4, R_vol = 5,
    R_velx = 6, R_vely = 7, R_velz = 8, R_wx = 9, R_wy = 10, R_wz = 11,
    R_bond_scale = 24
};
// intIdx (src/chemistry/bmx_chem.H:77-118)
enum {
    I_cell_type = 5, I_n_bnds = 6, I_seg1_id1 = 7, I_seg1_id2 = 11, I_site1 = 15,
    I_position = 19, I_fuse_flag = 20, I_split_flag = 21, I_new_flag = 22,
    I_fuse_tip = 25, I_dltd_site1 = 26, I_fix_site = 32, I_id = 33, I_cpu = 34
};

struct Layout {
    size_t stride, rdata, idata;
};

Layout layout_of(int nreal, int nint)
{
    Layout L;
    L.rdata = 3 * sizeof(double);
    L.idata = L.rdata + (size_t)nreal * sizeof(double) + 2 * sizeof(int);
    size_t end = L.idata + (size_t)nint * sizeof(int);
    L.stride = (end + 7) / 8 * 8;
    return L;
}

}  // namespace

extern "C" int bmxg_evolve_particles_aos(bmxg_ctx *ctx, void *particles, int64_t n, int32_t nreal,
                                         int32_t nint, const int64_t *colony_offsets, double dt,
                                         double *cost_per_colony, int32_t *nsubsteps)
{
    if (!ctx || n < 0 || (n > 0 && !particles)) return BMXG_ERR_ARG;
    if (nreal <= R_bond_scale || nint <= I_cpu) return BMXG_ERR_ARG;
    const Layout L = layout_of(nreal, nint);
    unsigned char *base = static_cast<unsigned char *>(particles);
    auto P = [&](int64_t i) { return reinterpret_cast<double *>(base + (size_t)i * L.stride); };
    auto R = [&](int64_t i) { return reinterpret_cast<double *>(base + (size_t)i * L.stride + L.rdata); };
    auto I = [&](int64_t i) { return reinterpret_cast<int *>(base + (size_t)i * L.stride + L.idata); };

    const size_t N = (size_t)n;
    std::vector<double> x(N), y(N), z(N), rad(N), len(N), th(N), ph(N), area(N), bs(N);
    std::vector<double> vx(N), vy(N), vz(N), wx(N), wy(N), wz(N);
    std::vector<int32_t> ct(N), id(N), cpu(N), nb(N), s1(4 * N), s2(4 * N), st(4 * N), pos(N), tip(N),
        fix(N), ff(N), sf(N), nf(N), dl(6 * N);
    bool rods = false;
    for (size_t i = 0; i < N; ++i) {
        const double *p = P(i), *r = R(i);
        const int *q = I(i);
        x[i] = p[0]; y[i] = p[1]; z[i] = p[2];
        rad[i] = r[R_radius]; len[i] = r[R_c_length]; th[i] = r[R_theta]; ph[i] = r[R_phi];
        area[i] = r[R_area]; bs[i] = r[R_bond_scale];
        vx[i] = r[R_velx]; vy[i] = r[R_vely]; vz[i] = r[R_velz];
        wx[i] = r[R_wx]; wy[i] = r[R_wy]; wz[i] = r[R_wz];
        ct[i] = q[I_cell_type]; id[i] = q[I_id]; cpu[i] = q[I_cpu]; nb[i] = q[I_n_bnds];
        for (int k = 0; k < 4; ++k) {
            s1[k * N + i] = q[I_seg1_id1 + k];
            s2[k * N + i] = q[I_seg1_id2 + k];
            st[k * N + i] = q[I_site1 + k];
        }
        for (int k = 0; k < 6; ++k) dl[k * N + i] = q[I_dltd_site1 + k];
        pos[i] = q[I_position]; tip[i] = q[I_fuse_tip]; fix[i] = q[I_fix_site];
        ff[i] = q[I_fuse_flag]; sf[i] = q[I_split_flag]; nf[i] = q[I_new_flag];
        rods |= (ct[i] == BMXG_FUNGI);
    }
    bmxg_particles s;
    std::memset(&s, 0, sizeof(s));
    s.n = n;
    s.x = x.data(); s.y = y.data(); s.z = z.data(); s.radius = rad.data(); s.cell_type = ct.data();
    s.velx = vx.data(); s.vely = vy.data(); s.velz = vz.data();
    s.wx = wx.data(); s.wy = wy.data(); s.wz = wz.data();
    s.fuse_flag = ff.data(); s.split_flag = sf.data(); s.new_flag = nf.data();
    if (rods) {
        s.c_length = len.data(); s.theta = th.data(); s.phi = ph.data(); s.area = area.data();
        s.bond_scale = bs.data(); s.id = id.data(); s.cpu = cpu.data(); s.n_bnds = nb.data();
        s.seg_id1 = s1.data(); s.seg_id2 = s2.data(); s.site = st.data(); s.position = pos.data();
        s.fuse_tip = tip.data(); s.fix_site = fix.data(); s.dltd = dl.data();
    }
    int rc = bmxg_set_state(ctx, &s, colony_offsets, BMXG_HOST);
    if (rc) return rc;
    rc = bmxg_evolve_particles(ctx, dt, cost_per_colony, nsubsteps);
    if (rc) return rc;
    rc = bmxg_get_state(ctx, &s, BMXG_HOST);
    if (rc) return rc;
    for (size_t i = 0; i < N; ++i) {
        double *p = P(i), *r = R(i);
        int *q = I(i);
        p[0] = x[i]; p[1] = y[i]; p[2] = z[i];
        r[R_velx] = vx[i]; r[R_vely] = vy[i]; r[R_velz] = vz[i];
        r[R_wx] = wx[i]; r[R_wy] = wy[i]; r[R_wz] = wz[i];
        q[I_fuse_flag] = ff[i]; q[I_split_flag] = sf[i]; q[I_new_flag] = nf[i];
        if (rods) {
            r[R_theta] = th[i]; r[R_phi] = ph[i];
            q[I_n_bnds] = nb[i];
            for (int k = 0; k < 4; ++k) {
                q[I_seg1_id1 + k] = s1[k * N + i];
                q[I_seg1_id2 + k] = s2[k * N + i];
                q[I_site1 + k] = st[k * N + i];
            }
            for (int k = 0; k < 6; ++k) q[I_dltd_site1 + k] = dl[k * N + i];
            q[I_position] = pos[i]; q[I_fix_site] = fix[i];
        }
    }
    return BMXG_OK;
}
