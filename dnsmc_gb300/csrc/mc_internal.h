// mc_internal.h -- data layout and kernel interface shared by the host runtime
// (mc_host.cpp) and the device code (mc_kernels.cu).
//
// Device layout (HBM):
//   field  : [f][i][k][j] with j fastest (the periodic axis the 32 lanes of a
//            packet tile), float T or float2 (T, x_H2O);
//   k table: [band][g][t][x] float, one contiguous nT*nX slice per spectral
//            sample (band, g) so a warp-uniform sample reads one slice;
//   Ib     : [band][t] float;  Ib_wall: [2][band] float (west, east);
//   tally  : [f][group][iR][kR][jR] double2 (sum X, sum X^2) over the rays of
//            one (cell, group) work item, j fastest so a packet stores 512
//            contiguous bytes.
#pragma once
#include <cstdint>

#include "../../include/dnsmc.h"

namespace dnsmc {

enum MarchMode { MODE_GREY = 0, MODE_T = 1, MODE_TX = 2 };

constexpr int kMaxLevels = 6;  // multigrid levels (grid_num)

// One alias-table entry of a spectral sample (band, g) inside a band group.
struct SpecEntry {
    float    prob;      // alias threshold (quantised to multiples of 2^-24)
    uint32_t alias_nb;  // alias index (low 16 bits) | band (high 16 bits)
    int32_t  koff;      // spectral sample index band*nq + g
    float    W;         // ray weight factor: w = W * k(T_i) * Ib(T_i)
};

// try_wait polls of a march's slab barrier before it gives up (each poll may
// suspend the thread for a while; the whole wait stays well under a second)
constexpr int kSlabWaitPolls = 1 << 16;

// Cells per lane of the fine-grid march (mc_march_pair.cuh): a packet is
// 32 * kLaneCells cells; the multigrid march uses 1.
constexpr int kLaneCells = 2;
// Bins per hemisphere of the tabulated surrogate of the control variate: the
// surrogate is stored at the nodes u = m / kSurBins of u = sqrt(|mu|) (mu the
// wall-normal direction cosine) and read by linear interpolation in u.
constexpr int kSurBins = 64;

struct MarchParams {
    // geometry: nw wall-normal cells (reference i), na (j) and nb (k) periodic
    int nw, na, nb;
    float da, db;             // periodic cell sizes
    const float *fw;          // nw+1 wall-normal faces
    // emission region (cells computed) and packet tiling
    int ew0, ew1, ea0, ea1, eb0, eb1;
    int tile_a, tile_b;       // tile_a * tile_b == 32
    int npa, npb, npw;        // packets along j, k, i
    int n_packets;            // npa * npb * npw
    int nfields;
    long long field_stride;   // cells per field (nw*na*nb)
    const float  *fieldT;     // MODE_GREY: temperature
    const int2   *fieldP;     // MODE_T: (ti, ft) table temperature cell and fraction
    const int4   *fieldPX;    // MODE_TX: (ti*(nX-1)+xi | ti<<16 ... see CellPos) per cell
    // spectral tables
    int nbands, nT, nX;
    float T0, invdT, X0, invdX;
    // per spectral sample (band*nq + g) one slab of slab_len float2: in the
    // first slab_klen the k entries [t < nT-1][x < nX-1] of two pairs each,
    // (k[t][x], k[t][x+1] - k[t][x]) and the same of row t+1, or the pairs
    // [t] (k[t], k[t+1] - k[t]); then the band's Ib pairs [t] (Ib[t], Ib[t+1]
    // - Ib[t]);
    // slab_len is even (16-byte rows).  Each warp copies its ray's slab into
    // shared memory: the march launches with warps * slab_len * 8 bytes.
    const float2 *slab;
    int slab_len, slab_klen;
    int slab_polls0;          // polls of the first wait for a slab copy: kSlabWaitPolls
                              // (fewer only in tests of the time-out path)
    const float *ibw;         // [2][band]
    const SpecEntry *entries;
    const int *group_start;   // n_tbins * n_groups + 1, temperature-bin major
    int n_groups;
    int n_tbins;              // 1: one table (at Tmax); nT: per table temperature
    // grey model
    float kappa;              // absorption coefficient
    float Wgrey;              // 4 * kappa * sigma
    float Tw4[2];             // wall T^4 (west, east), grey model
    // rays
    int rays;                 // rays per (cell, group) when rays_per_packet == 0
    const int *rays_per_packet;  // [G * rays_gstride + packet]
    int rays_gstride;         // 0: one count per packet for all groups; n_packets: per (group, packet)
    unsigned long long *item_steps;  // per item: ray-voxel steps summed over its rays, or null
    const unsigned int *item_order;  // queue position -> item (longest first), or null: natural order
    uint32_t key0, key1;      // Philox key (seed)
    int sampler;              // 0 iid Philox, 1 RQMC (shifted Sobol' net)
    int nbatch;               // RQMC replicates per item (rays divisible by it)
    uint32_t field_base;      // field index offset for the RNG counter
    float toll;
    float dtoll;              // ln(1/toll): optical-depth cut-off of the surrogate walk
    // general medium (GEN march): particles and grey walls
    const float *fieldV;      // [f][i][k][j] particle volume fraction, or null
    const float2 *part;       // [band] (absorption, scattering) per unit volume fraction [1/m], or null
    float fv_max;             // largest volume fraction of the fields (collision majorant)
    float hg_g;               // Henyey-Greenstein asymmetry factor
    float eps[2];             // wall emissivities (west, east)
    float W4sig;              // 4 sigma (grey model weight per unit absorption coefficient)
    // multigrid (MG march): after mg_steps steps a ray continues on the next
    // grid, 2x coarser per axis; level l has (nw, na, nb) >> l cells
    int mg_levels, mg_steps;
    const float *mgT;                  // coarse temperatures, level l at mg_off[l]: [f][i][k][j]
    const float *mgfw;                 // coarse wall-normal faces, level l at mg_fwoff[l]
    long long mg_off[kMaxLevels];
    int mg_fwoff[kMaxLevels];
    float mg_da[kMaxLevels], mg_db[kMaxLevels];  // periodic cell sizes per level
    float Ly, Lz;
    int max_steps;
    // work queue and outputs
    unsigned int *queue;      // atomic item counter (zeroed per launch)
    long long n_items;
    double2 *tally;           // see layout above
    long long region_cells;   // (ew1-ew0)*(ea1-ea0)*(eb1-eb0)
    unsigned int *status;     // DNSMC_STATUS_* bits
    unsigned long long *counters;  // [0] rays (lane-rays), [1] lane-steps
    // control variate: Y = the same ray through the layer-mean medium
    const float2 *sur;        // [f][sample][nw] (k_bar, Ib_bar) per layer
    const float4 *surtab;     // [f][sample][nw][2][kSurBins] surrogate per bin, see CvParams
    int n_samples;            // bands * nq (1 for the grey model)
    const float2 *beta;       // [f][group][iR][kR][jR] (beta_a, beta_b), or null: (1, -1)
    double *moments;          // [f][group][iR][kR][jR][9] per-ray moments (training solves)
    // trace (trace launches only)
    int trace_f, trace_g, trace_p, trace_r, trace_max;
    int *trace_rec;           // 6 words per step
    int *trace_n;
    unsigned int *trace_rng;
};

struct FinalizeParams {
    int nfields, n_groups;
    long long region_cells;
    int niR, njR, nkR;        // region extents (i, j, k)
    int tile_a, tile_b, npa, npb;
    int rays;
    const int *rays_per_packet;  // [g * rays_gstride + packet]
    int rays_gstride;
    int batched, nbatch;      // RQMC: variance from nbatch replicate means
    // reciprocals (1/N, 1/(N-1)) of the ray counts: per [g * rays_gstride +
    // packet] of rays_per_packet (device scratch, filled by launch_finalize),
    // of the uniform count and of nbatch (set by launch_finalize)
    double2 *rcp;
    double2 rcp_uniform, rcp_batch;
    const int *group_empty;   // 1 when the group has no emission
    const double2 *tally;
    const double2 *muY;       // (E[Y_a], E[Y_b]), tally layout, or null
    const float2 *beta;       // (beta_a, beta_b), tally layout, or null: (1, -1)
    double *Q;                // [f][cell] dense region, i fastest
    double *var;              // [f][cell]
    double *sigma;            // [f][cell]: sqrt(var)
    float *Qf;                // [f][cell] Q rounded to float, or nullptr
    float *sigf;              // [f][cell] sqrt(var * sig_scale) rounded to float (with Qf)
    double sig_scale;         // 1, or the drop-in's nVar / (nVar - 0.5) (code/mc_gpu.cu:221)
    double *Qg;               // [f][group][cell] or nullptr
    double *varg;             // [f][group][cell] or nullptr
    unsigned int *status;
};

// Entries of FinalizeParams::rcp: the indices g * rays_gstride + packet
// (rays_gstride 0: one count per packet for every group).
inline long long finalize_rcp_count(const FinalizeParams &f) {
    return (long long)(f.n_groups - 1) * f.rays_gstride + (long long)f.niR * f.npb * f.npa;
}

// A read-only view of a solver's device state for the control-variate
// network (mc_cvnet.cu); filled by solver_view (mc_host.cpp).
struct SolverView {
    int device;
    void *stream;
    int model, mode;                 // DNSMC_MODEL_*, MODE_*
    int imax, jmax, kmax, nfields, n_groups, nvar, sampler;
    int i0, i1, j0, j1, k0, k1;      // region
    int tile_a, tile_b, npa, npb, npw, n_packets;
    long long region_cells, field_stride;
    const float *fieldT;             // [f][i][k][j] (grey, T-only tables)
    const float2 *fieldTX;           // [f][i][k][j] (T, x_H2O)
    const float *fw;                 // wall-normal faces
    float T_lo, T_hi, X_lo, X_hi;    // table ranges (grey: 0, 0, 0, 0)
    // last solve (solved != 0)
    int solved, last_groups;
    const double *moments;           // [f][g][tc][9] or null
    const double *varg;              // [f][g][cell] dense i fastest
    const unsigned long long *item_steps;  // [f][g][packet]
    int rays;                        // uniform rays per (cell, group) when rays_item is null
    const int *rays_item;            // [g * rays_gstride + packet]
    int rays_gstride;
};
int solver_view(dnsmc_solver *s, SolverView *v);
// Device buffer of control-variate coefficients [f][g][tc] (tally order) that
// the next solve uses; the caller fills it on the solver's stream.
int solver_beta_device(dnsmc_solver *s, float2 **beta, long long *n);
// Device buffer of per-(group, packet) ray counts that the next solve uses.
int solver_rays_device(dnsmc_solver *s, int n_groups, int **rays);

// Rays per packet proportional to the packet's mean cell optical thickness
// kP(T, x) (dx dy dz)^(1/3), clamped and rounded to multiples of B.
struct AdaptParams {
    int nfields, nw, na, nb, mode;
    const float *fT;
    const float2 *fTX;
    const float *fw;
    float da, db;
    int ew0, ea0, eb0, njR, nkR, tile_a, tile_b, npa, npb, n_packets;
    long long field_stride;
    const float *kP;          // [nT][nX] Planck-mean absorption coefficient (null: grey kappa)
    int nT, nX;
    float T0, invdT, X0, invdX;
    float kappa;
    float per_tau;
    int B, nmin, nmax;
    int *rays;                // [packet]
};
int launch_adaptive_rays(const AdaptParams &a, void *stream);

// Table coordinates of a cell, computed once per solve (field_pos_kernel):
// p = clamp((v - v0)/dv, 0, n-1) split into cell i = min((int)p, n-2) and
// fraction p - i, for T and (MODE_TX) x_H2O.  MODE_TX packs
// {ti*(nX-1) + xi, ft, fx, ti} into an int4 (fractions as float bits), MODE_T
// {ti, ft} into an int2, so a march step needs no float-to-int split.
// Queue order of the march's items, longest first: a counting sort of the
// items by their ray count (n_items = nfields * n_groups * n_packets; rays of
// item (f, g, p) = rays[g * gstride + p]).  hist needs kOrderBuckets + 1 words.
constexpr int kOrderBuckets = 4096;
int launch_item_order(const int *rays, int gstride, int n_packets, int n_groups, long long n_items, int B,
                      unsigned int *hist, unsigned int *order, void *stream);

// One pass of the spline coarsening (interp3D, code/spline.cpp:35-116) over
// nlines = na * nb lines: line (la, lb) reads n fine values at
// src[(la*s_a + lb*s_b + (i-1)*s_e) * src_step] (positions xf[1..n]) and
// writes m coarse values at dst[la*d_a + lb*d_b + (c-1)*d_e] (positions
// xc[1..m]); work holds 3 * (n + 2) * nlines floats.
struct SplinePass {
    const float *src;
    long long s_a, s_b, s_e;
    int src_step;             // floats per source element (2: T of a (T, x) pair)
    float *dst;
    long long d_a, d_b, d_e;
    long long na, nlines;
    int n, m;
    const float *xf, *xc;     // 1-based device arrays of n + 2 and m + 2 floats
    float *work;
};
int launch_spline_pass(const SplinePass &q, void *stream);

// Kernels this library has launched in this process (every launch site
// calls note_launch; a CUDA-graph replay adds the kernel nodes of its graph).
void note_launch(long long n = 1);
long long launch_count();

// launchers (mc_kernels.cu); all stream-ordered
int launch_march_ex(int mode, const MarchParams &p, int blocks, int threads, void *stream, bool trace, bool cv,
                    bool mom, bool gen);
int march_occupancy_ex(int mode, int threads, bool cv, bool mom, bool gen, size_t smem);
int launch_march_mg(int mode, const MarchParams &p, int blocks, int threads, void *stream, bool trace);
int march_mg_occupancy(int mode, int threads, size_t smem);
// dynamic shared memory of a march launch with `cells` cells per lane: each
// warp's table slab (slab_len float2), then per thread and cell the three
// sums of the item (float pairs, 8 bytes), then per thread the RQMC replicate's shift (uint4)
inline size_t march_smem(const MarchParams &p, int threads, int cells) {
    return (size_t)((threads + 31) / 32) * (size_t)p.slab_len * 8u + (size_t)threads * (24u * (size_t)cells + 16u);
}
int launch_march_gen(int mode, const MarchParams &p, int blocks, int threads, void *stream, bool trace, bool cv,
                     bool mom);                                      // mc_march_gen.cu
int march_gen_occupancy(int mode, int threads, bool cv, bool mom, size_t smem);  // mc_march_gen.cu
int upload_sobol_dirs_gen(const uint32_t dirs[4][32]);               // mc_march_gen.cu
// the absorbing-gas march with two cells per lane (64-cell packets)    // mc_march_pair.cu
// (launch_march_gen: the same march with the general medium)
int launch_march_pair(int mode, const MarchParams &p, int blocks, int threads, void *stream, bool trace, bool cv,
                      bool mom);
int march_pair_occupancy(int mode, int threads, bool cv, bool mom, size_t smem);
int upload_sobol_dirs_pair(const uint32_t dirs[4][32]);
int launch_march(int mode, const MarchParams &p, int blocks, int threads,
                 void *stream, bool trace);
int launch_finalize(const FinalizeParams &p, void *stream);
int launch_field_pos(const float *fT, const float2 *fTX, int2 *outP, int4 *outPX, long long n, float T0,
                     float invdT, int nT, float X0, float invdX, int nX, void *stream);
// src element (i, j, k) at src[base + i*si + j*sj + k*sk]; writes dst[f] layout
int launch_pack_T(const float *src, float *dst, int nw, int na, int nb,
                  long long si, long long sj, long long sk, long long base,
                  void *stream);
int launch_pack_TX(const float *srcT, const float *srcX, float2 *dst, int nw,
                   int na, int nb, long long si, long long sj, long long sk,
                   long long base, void *stream);
// max T, min T, sum x and the count of non-positive or non-finite T over n
// cells into out[0..3] (device), deterministic
int launch_field_stats(const float *fT, const float2 *fTX, long long n,
                       double *partials, double *out, void *stream);
int field_stats_partials();   // doubles needed in `partials`
int march_occupancy(int mode, int threads);  // resident blocks per SM

// Control-variate preparation (all stream-ordered).
struct CvParams {
    int nfields, nw, na, nb;
    const float *fieldT;      // packed [f][i][k][j] (grey / T modes)
    const float2 *fieldTX;    // packed (T, x) (TX mode)
    int mode;                 // MODE_GREY / MODE_T / MODE_TX
    float2 *layer;            // [f][nw] (T_bar, x_bar)
    // tables (as MarchParams)
    int nbands, nq, nT, nX;
    float T0, invdT, X0, invdX;
    const float *ktab, *ibtab, *ibw;
    float kappa, Tw4[2];
    int n_samples;
    float2 *sur;              // [f][sample][nw]
    const float *fw;          // nw+1 faces
    float toll, dtoll;
    // [f][sample][nw][h][m]: the surrogate of a ray leaving the centre of
    // layer l into hemisphere h (0: towards the west wall, 1: east) with
    // sqrt(|mu|) = (m + r) / kSurBins, r in [0, 1), is
    //   J = J0 + r dJ (collected intensity), A = A0 + r dA (own-layer absorptance),
    // stored as (J0, dJ, A0, dA): the straight walk evaluated at the bin's two nodes
    float4 *surtab;
    double2 *Jhat;            // [f][sample][nw] (Jhat, Ahat): exact means of J and A over the
                              // isotropic directions (mu uniform on [-1, 1])
    float4 *Jf;               // [f][sample][nw] (Jhat hi, Jhat lo, Ahat, layer-mean Ib) for the mean
    // mean of Y per (field, group, cell) in tally layout
    int n_groups;
    const int *grp_start;     // n_groups+1 into samp_id / samp_C
    const int *samp_id;
    const double *samp_C;
    const float *samp_Cf;     // samp_C rounded to float
    double Wgrey;
    int ew0, ew1, ea0, ea1, eb0, eb1;
    long long region_cells;
    double2 *muY;
    // particles: absorption per unit volume fraction enters k of the cell and
    // of the layer-mean medium
    const float *fieldV;      // [f][i][k][j] volume fraction, or null
    const float2 *part;       // [band] (absorption, scattering) per unit volume fraction
    float *layerV;            // [f][nw] layer-mean volume fraction
    // node sums of E[Y] (tables without particles): per (field, group,
    // region layer) and table cell the sums over the group's samples, as
    // float pairs (hi, lo) of 8 bytes each; cv_node_count() of them
    double *nodes;
};
long long cv_node_count(const CvParams &c);
int launch_cv_prepare(const CvParams &c, void *stream);
constexpr int kCvMaxPlanes = 4096;  // wall-normal planes the control variate takes
int cv_table_allow_smem();          // once per device, before any launch_cv_prepare
int launch_cv_mean(const CvParams &c, void *stream);
int upload_sobol_dirs(const uint32_t dirs[4][32]);  // once per device
int device_sm_count();

}  // namespace dnsmc
