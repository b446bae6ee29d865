// k_noalloc.cu -- one FP64 sphere step that allocates no memory.
//
// Who needs it: code that may not call cudaMalloc on the step's path.  An
// AMReX application such as BMX hands all device memory out through its own
// arenas, sized up front, and a library that grabs memory behind them can
// make the arena's next allocation fail or fragment the device.  This entry
// point runs the same kernels as bmxg_step (binning, counting sort,
// k_sphere<FP64>) on arrays the caller owns, with the binning scratch taken
// from a fixed file-scope device array instead of from cudaMalloc.
//
// The array below is a static __device__ object: every GPU that loads the
// library holds it (kScratchBytes) until the process exits.  Its host-side
// name is only a stand-in for the symbol, never a device address: the first
// call on each device looks the address up with cudaGetSymbolAddress (with
// that device current) and caches it.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "../../include/bmxg.h"
#include "bmxg_kernels.cuh"

namespace bmxg {
namespace {

constexpr int kMaxN = 32768;       // particles per call
constexpr int kMaxCols = 65536;    // x-bins times y-bins per call
constexpr int kMaxDevices = 64;

// byte offsets of the scratch pieces (all 256-byte aligned)
constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kOffGeom = 0;
constexpr size_t kOffCnt = align256(kOffGeom + sizeof(DevGeom));
constexpr size_t kOffCol0 = align256(kOffCnt + sizeof(DevCounters));
constexpr size_t kOffCol1 = align256(kOffCol0 + sizeof(int) * kMaxN);
constexpr size_t kOffIz0 = align256(kOffCol1 + sizeof(int) * kMaxN);
constexpr size_t kOffIz1 = align256(kOffIz0 + sizeof(int) * kMaxN);
constexpr size_t kOffRel0 = align256(kOffIz1 + sizeof(int) * kMaxN);
constexpr size_t kOffRel1 = align256(kOffRel0 + sizeof(float4) * kMaxN);
constexpr size_t kOffPerm = align256(kOffRel1 + sizeof(float4) * kMaxN);
constexpr size_t kOffTmp = align256(kOffPerm + sizeof(int) * kMaxN);
constexpr size_t kOffOrig = align256(kOffTmp + sizeof(int) * kMaxN);
constexpr size_t kOffStart = align256(kOffOrig + sizeof(int) * kMaxN);
constexpr size_t kOffCount = align256(kOffStart + sizeof(int) * (kMaxCols + 1));
constexpr size_t kOffScan = align256(kOffCount + sizeof(int) * kMaxCols);
constexpr size_t kScratchBytes = align256(kOffScan + sizeof(int) * (kMaxCols / 4096 + 4));

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

__global__ void k_iota(int *a, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = i;
}

std::mutex g_mu;
unsigned char *g_addr[kMaxDevices] = {nullptr};

// device address of g_scratch on the current device (looked up once per device)
int scratch_address(unsigned char **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return BMXG_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return BMXG_ERR_CUDA;
        g_addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_addr[dev];
    return BMXG_OK;
}

}  // namespace
}  // namespace bmxg

using namespace bmxg;

extern "C" int bmxg_sphere_step_noalloc(const bmxg_params *params, const bmxg_geometry *geom, int64_t n,
                                        const double *x, const double *y, const double *z,
                                        const double *radius, double *x_out, double *y_out, double *z_out,
                                        double *vel_x, double *vel_y, double *vel_z, double dt, void *stream,
                                        int64_t *n_out_of_domain)
{
    (void)cudaGetLastError();  // a non-sticky error another library left on this thread is not ours
    if (n_out_of_domain) *n_out_of_domain = 0;
    if (!params || !geom || n < 0) return BMXG_ERR_ARG;
    // sizes first: beyond the fixed scratch is BMXG_ERR_CAPACITY, whatever else is wrong
    if (n > kMaxN) return BMXG_ERR_CAPACITY;                      // more than 32768 particles
    const int64_t ncols = (int64_t)geom->n_cell[0] * geom->n_cell[1];
    if (ncols > kMaxCols) return BMXG_ERR_CAPACITY;               // more than 65536 columns
    if (n > 0 && (!x || !y || !z || !radius || !x_out || !y_out || !z_out || !vel_x || !vel_y || !vel_z))
        return BMXG_ERR_ARG;
    for (int d = 0; d < 3; ++d) {
        if (!(geom->prob_hi[d] > geom->prob_lo[d]) || geom->n_cell[d] < 1) return BMXG_ERR_ARG;
        if (geom->is_periodic[d] && geom->n_cell[d] < 3) return BMXG_ERR_UNSUPPORTED;
    }
    if (geom->is_periodic[2]) return BMXG_ERR_UNSUPPORTED;
    unsigned char *base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    if (n == 0) return BMXG_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    // the colony geometry, as the context builds it
    DevGeom G;
    std::memset(&G, 0, sizeof(G));
    double diag2 = 0.0;
    for (int d = 0; d < 3; ++d) {
        G.plo[d] = geom->prob_lo[d];
        G.phi[d] = geom->prob_hi[d];
        G.len[d] = geom->prob_hi[d] - geom->prob_lo[d];
        G.n[d] = geom->n_cell[d];
        G.dx[d] = G.len[d] / (double)G.n[d];
        G.dxi[d] = 1.0 / G.dx[d];
        G.dxf[d] = (float)G.dx[d];
        G.per[d] = geom->is_periodic[d] ? 1 : 0;
        diag2 += 4.0 * G.dx[d] * G.dx[d];
    }
    G.col_base = 0;
    G.slot_base = 0;
    G.slot_end = (int)n;
    G.nbh_trivial = (params->neighborhood >= diag2 * (1.0 + 1e-9)) ? 1 : 0;

    DevState S;
    std::memset(&S, 0, sizeof(S));
    S.n = (int)n;
    S.ncol = 1;
    S.ncols_total = (int)ncols;
    S.geoms = reinterpret_cast<DevGeom *>(base + kOffGeom);
    S.cnt = reinterpret_cast<DevCounters *>(base + kOffCnt);
    S.x[0] = const_cast<double *>(x);
    S.y[0] = const_cast<double *>(y);
    S.z[0] = const_cast<double *>(z);
    S.x[1] = x_out;
    S.y[1] = y_out;
    S.z[1] = z_out;
    S.col[0] = reinterpret_cast<int *>(base + kOffCol0);
    S.col[1] = reinterpret_cast<int *>(base + kOffCol1);
    S.iz[0] = reinterpret_cast<int *>(base + kOffIz0);
    S.iz[1] = reinterpret_cast<int *>(base + kOffIz1);
    S.rel[0] = reinterpret_cast<float4 *>(base + kOffRel0);
    S.rel[1] = reinterpret_cast<float4 *>(base + kOffRel1);
    S.perm[0] = reinterpret_cast<int *>(base + kOffPerm);
    S.tmp = reinterpret_cast<int *>(base + kOffTmp);
    S.orig = reinterpret_cast<int *>(base + kOffOrig);
    S.colstart[0] = reinterpret_cast<int *>(base + kOffStart);
    S.colcnt = reinterpret_cast<int *>(base + kOffCount);
    S.rad = const_cast<double *>(radius);
    S.vx = vel_x;
    S.vy = vel_y;
    S.vz = vel_z;
    int *scan = reinterpret_cast<int *>(base + kOffScan);

    // every call reuses the same scratch: clear what must start at zero
    if (cudaMemcpyAsync(base + kOffGeom, &G, sizeof(G), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(base + kOffCnt, 0, sizeof(DevCounters), st) != cudaSuccess ||
        cudaMemsetAsync(S.colcnt, 0, sizeof(int) * ncols, st) != cudaSuccess)
        return BMXG_ERR_CUDA;
    const int block = 256;
    const int grid = (int)std::min<int64_t>((n + block - 1) / block, 4096);
    k_iota<<<grid, block, 0, st>>>(S.orig, (int)n);
    const DevParams P{params->bndry_width, params->stiffness,     params->z_wall,      params->z_bndry_width,
                      params->z_stiffness,  params->z_gravity,     params->bond_strength, params->bond_cutoff,
                      params->viscosity,    params->neighborhood};
    launch_bin(S, 0, grid, block, st);
    launch_rebuild(S, 0, scan, grid, block, st);
    launch_sphere_step(S, P, dt / 1.0, 0, BMXG_FP64_FORM, grid, block, st);
    if (cudaGetLastError() != cudaSuccess) return BMXG_ERR_CUDA;  // a launch failed
    DevCounters h;
    if (cudaMemcpyAsync(&h, base + kOffCnt, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess) return BMXG_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return BMXG_ERR_CUDA;
    if (n_out_of_domain) *n_out_of_domain = (int64_t)h.out_of_domain;
    // as bmxg_step: inconsistent counting-sort counts are an internal error
    if (h.bad_index) return BMXG_ERR_STATE;
    if (h.nonfinite) return BMXG_ERR_NONFINITE;
    return BMXG_OK;
}
