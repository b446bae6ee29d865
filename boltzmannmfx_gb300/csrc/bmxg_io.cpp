// bmxg_io.cpp -- fixture I/O of the particle state (host only).
//
//  * bmxg_read_ascii / bmxg_write_ascii: the particle input format of
//    BMXParticleContainer::InitParticlesAscii (src/des/bmx_pc_init.cpp:17-132):
//    the particle count, then 27 whitespace-separated values per particle
//    (position, radius, c_length, theta, phi, area, vol, velocity, angular
//    velocity, force, torque, gradient, dadt, dvdt, cell_type), read as one
//    stream like the reference does (line breaks carry no meaning).
//  * bmxg_write_vtk: the legacy-VTK polydata of
//    BMXParticleContainer::WriteToAscii (src/des/bmx_pc_write.cpp:11-219):
//    two end points per segment, one two-vertex polygon per particle, the
//    particle index as cell scalar and a concentration as point scalar.
//  * bmxg_read_checkpoint: the particles of an AMReX checkpoint in the
//    Version_Two_Dot_One_double format that bmx::WriteCheckPointFile writes
//    (src/io/bmx_chk.cpp:114-160; read back by bmx::Restart,
//    src/io/bmx_restart.cpp:24-225): a text Header, then per grid a block of
//    (2 + n_int) int32 per particle (AMReX's packed id/cpu, then the integer
//    components) followed by (3 + n_real) doubles (position, then the real
//    components), in the byte order of the writing host.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "bmxg.h"

namespace {

constexpr double kPi = 3.14159265358979323846;

thread_local std::string g_io_err;

int io_fail(int code, const std::string &msg)
{
    g_io_err = msg;
    return code;
}

// Field positions of one particle-component layout.  -1: not stored in that
// layout (the reader fills the reference's default instead).
struct Layout {
    int n_real, n_int;
    int radius, c_length, theta, phi, area, vol, vel[3], w[3], bond_scale;
    int cell_type, n_bnds, seg_id1, seg_id2, site, position, fuse_flag, split_flag, new_flag, fuse_tip, dltd,
        fix_site, id, cpu;
};

// realIdx / intIdx of src/chemistry/bmx_chem.H:38-118 (MAX_CHEM_REAL_VAR 34,
// MAX_CHEM_INT_VAR 35).
constexpr Layout kCurrent = {34, 35, 0, 1, 2, 3, 4, 5, {6, 7, 8}, {9, 10, 11}, 24,
                             5,  6,  7, 11, 15, 19, 20, 21, 22, 25, 26, 32, 33, 34};
// The 33 + 33 components of the checkpoints shipped with the reference
// (exec/fungi/chk357900, AMReX 22.03): realIdx without bond_scale (its
// components 0..23 are the current ones, then the chemistry block), intIdx
// without fuse_tip and fix_site (components 0..24 as now, the six dltd_*
// at 25..30, id and cpu at 31 and 32).
constexpr Layout kLegacy33 = {33, 33, 0, 1, 2, 3, 4, 5, {6, 7, 8}, {9, 10, 11}, -1,
                              5,  6,  7, 11, 15, 19, 20, 21, 22, -1, 25, -1, 31, 32};

const Layout *layout_for(int n_real, int n_int)
{
    if (n_real == kCurrent.n_real && n_int == kCurrent.n_int) return &kCurrent;
    if (n_real == kLegacy33.n_real && n_int == kLegacy33.n_int) return &kLegacy33;
    return nullptr;
}

template <class T>
void put(T *dst, int64_t i, T v)
{
    if (dst) dst[i] = v;
}

template <class T>
void put_plane(T *dst, int64_t n, int k, int64_t i, T v)
{
    if (dst) dst[(size_t)k * n + i] = v;
}

// Reference defaults of InitParticlesAscii for fields the file does not carry.
void defaults(bmxg_particles *p, int64_t i, int64_t n)
{
    put(p->bond_scale, i, 1.0);
    put(p->fuse_tip, i, 0);
    put(p->cpu, i, 0);
    put(p->id, i, (int32_t)(i + 1));  // ParticleType::NextID() starts at 1
    put(p->n_bnds, i, 0);
    put(p->position, i, 0);
    put(p->fix_site, i, 0);
    put(p->fuse_flag, i, 0);
    put(p->split_flag, i, 0);
    put(p->new_flag, i, 0);
    for (int k = 0; k < 4; ++k) {
        put_plane(p->seg_id1, n, k, i, 0);
        put_plane(p->seg_id2, n, k, i, 0);
        put_plane(p->site, n, k, i, 0);
    }
    for (int k = 0; k < 6; ++k) put_plane(p->dltd, n, k, i, 0);
}

}  // namespace

extern "C" {

const char *bmxg_io_last_error(void) { return g_io_err.c_str(); }

int bmxg_read_ascii(const char *path, bmxg_particles *out, int64_t cap, int64_t *n_out)
{
    if (!path || !n_out) return io_fail(BMXG_ERR_ARG, "path and n are required");
    *n_out = 0;
    std::ifstream in(path);
    if (!in.good()) return io_fail(BMXG_ERR_ARG, std::string("cannot open ") + path);
    long long np = -1;
    in >> np;
    if (!in.good() || np < 0) return io_fail(BMXG_ERR_ARG, "cannot read the particle count (first value)");
    *n_out = np;
    if (!out || cap < np) return io_fail(BMXG_ERR_CAPACITY, "buffer smaller than the particle count");
    if (out->n != np) return io_fail(BMXG_ERR_ARG, "out->n must equal the particle count");
    const int64_t n = out->n;
    for (int64_t i = 0; i < np; ++i) {
        double v[26];
        int ct = 0;
        for (double &x : v) in >> x;
        in >> ct;
        if (in.fail()) return io_fail(BMXG_ERR_ARG, "file ends or is malformed at particle " + std::to_string(i));
        defaults(out, i, n);
        put(out->x, i, v[0]);
        put(out->y, i, v[1]);
        put(out->z, i, v[2]);
        put(out->radius, i, v[3]);
        put(out->c_length, i, v[4]);
        put(out->theta, i, v[5]);
        put(out->phi, i, v[6]);
        put(out->area, i, v[7]);
        // v[8] vol, v[15..25] force, torque, gradient, dadt, dvdt: not step state
        put(out->velx, i, v[9]);
        put(out->vely, i, v[10]);
        put(out->velz, i, v[11]);
        put(out->wx, i, v[12]);
        put(out->wy, i, v[13]);
        put(out->wz, i, v[14]);
        put(out->cell_type, i, (int32_t)ct);
    }
    return BMXG_OK;
}

int bmxg_write_ascii(const char *path, const bmxg_particles *p)
{
    if (!path || !p || p->n < 0 || !p->x || !p->y || !p->z || !p->radius || !p->cell_type)
        return io_fail(BMXG_ERR_ARG, "path, x, y, z, radius and cell_type are required");
    FILE *f = std::fopen(path, "w");
    if (!f) return io_fail(BMXG_ERR_ARG, std::string("cannot open ") + path + ": " + std::strerror(errno));
    auto g = [&](const double *a, int64_t i) { return a ? a[i] : 0.0; };
    std::fprintf(f, "%lld\n", (long long)p->n);
    for (int64_t i = 0; i < p->n; ++i) {
        const double r = p->radius[i];
        const double L = g(p->c_length, i);
        // vol is not step state; written as the reference's shapes would have it
        const double vol = (p->cell_type[i] == BMXG_FUNGI) ? kPi * r * r * L : 4.0 / 3.0 * kPi * r * r * r;
        std::fprintf(f, "%.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g", p->x[i], p->y[i], p->z[i], r, L,
                     g(p->theta, i), g(p->phi, i), g(p->area, i), vol);
        std::fprintf(f, " %.17g %.17g %.17g %.17g %.17g %.17g", g(p->velx, i), g(p->vely, i), g(p->velz, i),
                     g(p->wx, i), g(p->wy, i), g(p->wz, i));
        std::fprintf(f, " 0 0 0 0 0 0 0 0 0 0 0 %d\n", (int)p->cell_type[i]);
    }
    const bool ok = !std::ferror(f);
    std::fclose(f);
    return ok ? BMXG_OK : io_fail(BMXG_ERR_ARG, "write failed");
}

int bmxg_write_vtk(const char *path, const bmxg_particles *p, const double *conc_b)
{
    if (!path || !p || p->n < 0 || !p->x || !p->y || !p->z)
        return io_fail(BMXG_ERR_ARG, "path, x, y and z are required");
    std::ofstream f(path);
    if (!f.good()) return io_fail(BMXG_ERR_ARG, std::string("cannot open ") + path);
    const int64_t n = p->n;
    const int npc = 2;  // vertices per particle
    f << "# vtk DataFile Version 3.0 \nhexagon using polygon function vtk \nASCII\nDATASET POLYDATA\n \n";
    f << "POINTS " << npc * n << " float\n";
    f.precision(8);
    for (int64_t i = 0; i < n; ++i) {
        const double L = p->c_length ? p->c_length[i] : 0.0;
        const double th = p->theta ? p->theta[i] : 0.0, ph = p->phi ? p->phi[i] : 0.0;
        const double nx = std::sin(th) * std::cos(ph), ny = std::sin(th) * std::sin(ph), nz = std::cos(th);
        f << p->x[i] + 0.5 * nx * L << " " << p->y[i] + 0.5 * ny * L << " " << p->z[i] + 0.5 * nz * L << "\n";
        f << p->x[i] - 0.5 * nx * L << " " << p->y[i] - 0.5 * ny * L << " " << p->z[i] - 0.5 * nz * L << "\n \n";
    }
    f << "POLYGONS " << n << " " << (npc + 1) * n << "\n";
    for (int64_t i = 0; i < n; ++i) f << npc << " " << i * npc << " " << i * npc + 1 << " \n";
    f << " \nCELL_DATA " << n << "\nPOINT_DATA " << npc * n << "\nSCALARS cell int\nLOOKUP_TABLE default\n";
    for (int64_t i = 0; i < n; ++i) f << i << " " << i << " \n";
    f << "\nSCALARS conc_B float\nLOOKUP_TABLE default\n";
    for (int64_t i = 0; i < n; ++i) {
        const double c = conc_b ? conc_b[i] : 0.0;
        f << c << " " << c << "\n";
    }
    f.flush();
    return f.good() ? BMXG_OK : io_fail(BMXG_ERR_ARG, "write failed");
}

int bmxg_read_checkpoint(const char *dir, int32_t level, bmxg_particles *out, int64_t cap, int64_t *n_out)
{
    if (!dir || !n_out) return io_fail(BMXG_ERR_ARG, "dir and n are required");
    *n_out = 0;
    const std::string base(dir);
    std::ifstream hdr(base + "/Header");
    if (!hdr.good()) return io_fail(BMXG_ERR_ARG, "cannot open " + base + "/Header");
    std::string version;
    int dim = 0, n_real = 0, n_int = 0, is_chk = 0, finest = -1;
    long long np_total = 0, next_id = 0;
    hdr >> version >> dim >> n_real;
    if (version != "Version_Two_Dot_One_double")
        return io_fail(BMXG_ERR_UNSUPPORTED, "particle file version " + version + " (only Version_Two_Dot_One_double)");
    if (dim != 3) return io_fail(BMXG_ERR_UNSUPPORTED, "dimension " + std::to_string(dim));
    std::string name;
    for (int k = 0; k < n_real; ++k) hdr >> name;
    hdr >> n_int;
    for (int k = 0; k < n_int; ++k) hdr >> name;
    hdr >> is_chk >> np_total >> next_id >> finest;
    if (hdr.fail() || finest < 0) return io_fail(BMXG_ERR_ARG, "malformed particle Header");
    if (!is_chk) return io_fail(BMXG_ERR_UNSUPPORTED, "not a checkpoint (integer components missing)");
    const Layout *L = layout_for(n_real, n_int);
    if (!L)
        return io_fail(BMXG_ERR_UNSUPPORTED, "component layout " + std::to_string(n_real) + " real / " +
                                                 std::to_string(n_int) + " int");
    std::vector<int> ngrids(finest + 1);
    for (int &g : ngrids) hdr >> g;
    struct Grid {
        int lev, which;
        long long count, where;
    };
    std::vector<Grid> grids;
    for (int lev = 0; lev <= finest; ++lev)
        for (int g = 0; g < ngrids[lev]; ++g) {
            Grid gr{lev, 0, 0, 0};
            hdr >> gr.which >> gr.count >> gr.where;
            if (gr.count > 0 && (level < 0 || level == lev)) grids.push_back(gr);
        }
    if (hdr.fail()) return io_fail(BMXG_ERR_ARG, "malformed grid table in the particle Header");
    long long np = 0;
    for (const Grid &g : grids) np += g.count;
    *n_out = np;
    if (!out || cap < np) return io_fail(BMXG_ERR_CAPACITY, "buffer smaller than the particle count");
    if (out->n != np) return io_fail(BMXG_ERR_ARG, "out->n must equal the particle count");
    const int64_t n = out->n;
    int64_t i = 0;
    std::vector<int32_t> iv;
    std::vector<double> rv;
    for (const Grid &g : grids) {
        char fn[64];
        std::snprintf(fn, sizeof(fn), "/Level_%d/DATA_%05d", g.lev, g.which);
        std::ifstream d(base + fn, std::ios::binary);
        if (!d.good()) return io_fail(BMXG_ERR_ARG, "cannot open " + base + fn);
        d.seekg(g.where);
        const size_t ni = (size_t)g.count * (2 + n_int), nr = (size_t)g.count * (3 + n_real);
        iv.resize(ni);
        rv.resize(nr);
        d.read((char *)iv.data(), (std::streamsize)(ni * sizeof(int32_t)));
        d.read((char *)rv.data(), (std::streamsize)(nr * sizeof(double)));
        if (!d.good()) return io_fail(BMXG_ERR_ARG, std::string("short read in ") + base + fn);
        for (long long q = 0; q < g.count; ++q, ++i) {
            const int32_t *ip = &iv[(size_t)q * (2 + n_int) + 2];
            const double *rp = &rv[(size_t)q * (3 + n_real)];
            const double *rc = rp + 3;
            defaults(out, i, n);
            put(out->x, i, rp[0]);
            put(out->y, i, rp[1]);
            put(out->z, i, rp[2]);
            put(out->radius, i, rc[L->radius]);
            put(out->c_length, i, rc[L->c_length]);
            put(out->theta, i, rc[L->theta]);
            put(out->phi, i, rc[L->phi]);
            put(out->area, i, rc[L->area]);
            put(out->velx, i, rc[L->vel[0]]);
            put(out->vely, i, rc[L->vel[1]]);
            put(out->velz, i, rc[L->vel[2]]);
            put(out->wx, i, rc[L->w[0]]);
            put(out->wy, i, rc[L->w[1]]);
            put(out->wz, i, rc[L->w[2]]);
            if (L->bond_scale >= 0) put(out->bond_scale, i, rc[L->bond_scale]);
            put(out->cell_type, i, ip[L->cell_type]);
            put(out->n_bnds, i, ip[L->n_bnds]);
            for (int k = 0; k < 4; ++k) {
                put_plane(out->seg_id1, n, k, i, ip[L->seg_id1 + k]);
                put_plane(out->seg_id2, n, k, i, ip[L->seg_id2 + k]);
                put_plane(out->site, n, k, i, ip[L->site + k]);
            }
            put(out->position, i, ip[L->position]);
            put(out->fuse_flag, i, ip[L->fuse_flag]);
            put(out->split_flag, i, ip[L->split_flag]);
            put(out->new_flag, i, ip[L->new_flag]);
            if (L->fuse_tip >= 0) put(out->fuse_tip, i, ip[L->fuse_tip]);
            for (int k = 0; k < 6; ++k) put_plane(out->dltd, n, k, i, ip[L->dltd + k]);
            if (L->fix_site >= 0) put(out->fix_site, i, ip[L->fix_site]);
            put(out->id, i, ip[L->id]);
            put(out->cpu, i, ip[L->cpu]);
        }
    }
    return BMXG_OK;
}

}  // extern "C"
