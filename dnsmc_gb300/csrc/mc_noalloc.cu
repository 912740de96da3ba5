// mc_noalloc.cu -- grey-medium solve that allocates no device memory.
//
// Some host codes cannot call cudaMalloc at solve time: a DNS that hands all
// free device memory to its own pool allocator at start-up (a new allocation
// then fails or fragments the pool), or production runs that forbid any
// allocation after initialisation so their memory footprint stays fixed.
// dnsmc_solve_grey_noalloc serves them: the caller passes device input and
// output arrays, and every intermediate buffer of the solve (packed field,
// wall-normal faces, per-cell tallies, work-queue counter, status and counter
// words) lives in g_noalloc_scratch, one file-scope __device__ array of fixed
// size that each GPU loading this library holds until the process exits.
//
// The kernels are the same persistent march and finalize kernels the handle
// API launches (launch_march / launch_finalize / launch_pack_T in
// mc_kernels.cu); only the location of their scratch differs.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/dnsmc.h"
#include "mc_internal.h"

namespace dnsmc {

int report_error(int code, const char *msg);  // mc_host.cpp: sets dnsmc_last_error()

namespace {

constexpr long long kMaxCells = DNSMC_NOALLOC_MAX_CELLS;
constexpr int kMaxFaces = DNSMC_NOALLOC_MAX_IMAX + 1;
constexpr size_t kTallyOff = 0;                                      // double2 per cell
constexpr size_t kFieldOff = kTallyOff + (size_t)kMaxCells * 16;     // float per cell
constexpr size_t kFacesOff = kFieldOff + (size_t)kMaxCells * 4;      // wall-normal faces
constexpr size_t kMiscOff = kFacesOff + (((size_t)kMaxFaces * 4 + 255) / 256) * 256;
constexpr size_t kMiscBytes = 256;  // [0] queue, [1] status, [2] group flag (uint32); [2..3] counters (u64)
constexpr size_t kScratchBytes = kMiscOff + kMiscBytes;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of g_noalloc_scratch per device.  In host code the symbol
// names a host-side stand-in, so the address is looked up once per device
// with that device current and passed to the kernels.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char *g_addr[kMaxDevices] = {};

int scratch_address(unsigned char **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return report_error(DNSMC_ERR_NODEVICE, "no current CUDA device");
    if (dev < 0 || dev >= kMaxDevices) return report_error(DNSMC_ERR_ARG, "device index beyond 63");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            char msg[160];
            snprintf(msg, sizeof msg, "cudaGetSymbolAddress(g_noalloc_scratch) failed: %s", cudaGetErrorString(e));
            return report_error(DNSMC_ERR_CUDA, msg);
        }
        g_addr[dev] = (unsigned char *)p;
    }
    *out = g_addr[dev];
    return DNSMC_OK;
}

}  // namespace
}  // namespace dnsmc

using namespace dnsmc;

extern "C" int dnsmc_solve_grey_noalloc(const dnsmc_config *cfg, const float *xu, const float *dT, double *dQ,
                                        double *dvar, uint32_t *dstatus, void *stream) {
    if (!cfg || !xu || !dT || !dQ || !dvar) return report_error(DNSMC_ERR_ARG, "null argument");
    const dnsmc_config &c = *cfg;
    if (c.model != DNSMC_MODEL_GREY) return report_error(DNSMC_ERR_ARG, "the allocation-free solve is grey only");
    if (c.imax < 1 || c.jmax < 1 || c.kmax < 1) return report_error(DNSMC_ERR_ARG, "imax, jmax, kmax must be >= 1");
    const long long ncell = (long long)c.imax * c.jmax * c.kmax;
    if (ncell > kMaxCells || c.imax > DNSMC_NOALLOC_MAX_IMAX) {
        char msg[200];
        snprintf(msg, sizeof msg,
                 "grid %dx%dx%d exceeds the allocation-free limit (at most %d cells and imax <= %d)", c.imax,
                 c.jmax, c.kmax, DNSMC_NOALLOC_MAX_CELLS, DNSMC_NOALLOC_MAX_IMAX);
        return report_error(DNSMC_ERR_ARG, msg);
    }
    if (c.grid_num != 1) return report_error(DNSMC_ERR_ARG, "grid_num must be 1");
    if (c.sampler != DNSMC_SAMPLER_IID) return report_error(DNSMC_ERR_ARG, "the allocation-free solve uses the IID sampler");
    if (c.nvar < 1 || c.photmax < 1) return report_error(DNSMC_ERR_ARG, "nvar and photmax must be >= 1");
    if (!(c.toll > 0) || c.toll >= 1) return report_error(DNSMC_ERR_ARG, "toll must be in (0, 1)");
    // the march counts crossings in FP32, exact below 2^22 (as the handle API)
    if (c.max_steps < 1 || c.max_steps > (1 << 22))
        return report_error(DNSMC_ERR_ARG, "max_steps must be in [1, 4194304]");
    if (!(c.eps_west == 1.0f) || !(c.eps_east == 1.0f)) return report_error(DNSMC_ERR_ARG, "walls must be black");
    if (!(c.kappa >= 0) || !(c.T_west >= 0) || !(c.T_east >= 0)) return report_error(DNSMC_ERR_ARG, "bad kappa or wall T");
    if (!(c.Ly > 0) || !(c.Lz > 0)) return report_error(DNSMC_ERR_ARG, "Ly and Lz must be > 0");
    if (c.block_threads && c.block_threads != 128 && c.block_threads != 256)
        return report_error(DNSMC_ERR_ARG, "block_threads must be 0, 128 or 256");
    if (c.tile_a && c.tile_a != 8 && c.tile_a != 16 && c.tile_a != 32)
        return report_error(DNSMC_ERR_ARG, "tile_a must be 0, 8, 16 or 32");
    const long long rays = (long long)c.nvar * c.photmax;
    if (rays > 0x7fffffffLL) return report_error(DNSMC_ERR_ARG, "too many rays per cell");

    unsigned char *base = nullptr;
    if (int rc = scratch_address(&base)) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    float *field = (float *)(base + kFieldOff);
    float *faces = (float *)(base + kFacesOff);
    unsigned int *misc = (unsigned int *)(base + kMiscOff);
    unsigned long long *counters = (unsigned long long *)(base + kMiscOff + 16);
    double2 *tally = (double2 *)(base + kTallyOff);

    // Scratch keeps the previous call's contents: the queue, status, group
    // flag and counters must start at zero; faces, field and tallies are
    // fully overwritten below before they are read.
    cudaError_t e = cudaMemsetAsync(misc, 0, kMiscBytes, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(faces, xu, (size_t)(c.imax + 1) * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return report_error(DNSMC_ERR_CUDA, cudaGetErrorString(e));
    int rc = launch_pack_T(dT, field, c.imax, c.jmax, c.kmax, 1, c.imax, (long long)c.imax * c.jmax, 0, st);
    if (rc) return report_error(DNSMC_ERR_CUDA, cudaGetErrorString((cudaError_t)rc));

    // the grey black-wall march runs kLaneCells cells per lane
    // the handle API's automatic packet shape (8 x 8, or 16 x 4 / 32 x 2 for
    // fewer than 8 / 4 cells along k)
    const int ta = c.tile_a ? c.tile_a : (c.kmax >= 8 ? 8 : (c.kmax >= 4 ? 16 : 32));
    const int tb = 32 / ta * kLaneCells;
    MarchParams P{};
    P.nw = c.imax; P.na = c.jmax; P.nb = c.kmax;
    P.da = c.Ly / (float)c.jmax; P.db = c.Lz / (float)c.kmax;
    P.fw = faces;
    P.ew0 = 0; P.ew1 = c.imax; P.ea0 = 0; P.ea1 = c.jmax; P.eb0 = 0; P.eb1 = c.kmax;
    P.tile_a = ta; P.tile_b = tb;
    P.npa = (c.jmax + ta - 1) / ta; P.npb = (c.kmax + tb - 1) / tb; P.npw = c.imax;
    P.n_packets = P.npa * P.npb * P.npw;
    P.nfields = 1;
    P.field_stride = ncell;
    P.fieldT = field;
    P.n_groups = 1;
    P.n_tbins = 1;
    P.kappa = c.kappa;
    P.Wgrey = (float)(4.0 * c.kappa * 5.670373e-08);
    P.Tw4[0] = c.T_west * c.T_west * c.T_west * c.T_west;
    P.Tw4[1] = c.T_east * c.T_east * c.T_east * c.T_east;
    P.rays = (int)rays;
    P.key0 = (uint32_t)(c.seed & 0xffffffffu);
    P.key1 = (uint32_t)(c.seed >> 32);
    P.sampler = DNSMC_SAMPLER_IID;
    P.nbatch = c.nvar;
    P.toll = c.toll;
    P.dtoll = (float)(-log((double)c.toll));
    P.max_steps = c.max_steps;
    P.slab_polls0 = kSlabWaitPolls;  // grey: no table slab is copied
    P.queue = misc;
    P.status = misc + 1;
    P.counters = counters;
    P.region_cells = ncell;
    P.n_items = P.n_packets;
    P.tally = tally;
    const int threads = c.block_threads ? c.block_threads : 256;
    // persistent grid: resident blocks at the launch's dynamic shared memory
    const size_t smem = march_smem(P, threads, kLaneCells);
    const int blocks = device_sm_count() * march_occupancy_ex(MODE_GREY, threads, false, false, false, smem);
    rc = launch_march(MODE_GREY, P, blocks > 0 ? blocks : 1, threads, st, false);
    if (rc) return report_error(DNSMC_ERR_CUDA, cudaGetErrorString((cudaError_t)rc));

    FinalizeParams F{};
    F.nfields = 1; F.n_groups = 1; F.region_cells = ncell;
    F.niR = c.imax; F.njR = c.jmax; F.nkR = c.kmax;
    F.tile_a = ta; F.tile_b = tb; F.npa = P.npa; F.npb = P.npb;
    F.rays = (int)rays;
    F.batched = 0; F.nbatch = c.nvar;
    F.group_empty = (const int *)(misc + 2);
    F.tally = tally;
    F.Q = dQ; F.var = dvar;
    F.status = misc + 1;
    rc = launch_finalize(F, st);
    if (rc) return report_error(DNSMC_ERR_CUDA, cudaGetErrorString((cudaError_t)rc));
    // the status bits of this solve (bad temperature, step cap, non-finite
    // contribution) into the caller's word: a device-to-device copy on the
    // stream, after the finalize
    if (dstatus) {
        e = cudaMemcpyAsync(dstatus, misc + 1, sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return report_error(DNSMC_ERR_CUDA, cudaGetErrorString(e));
    }
    return DNSMC_OK;
}
