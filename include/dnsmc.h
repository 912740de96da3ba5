/*
 * dnsmc.h -- C ABI of the GB300 reverse Monte Carlo radiative-source solver.
 *
 * Two layers:
 *
 *  1. The reference drop-in pair  mc_gpu_ / get_results_.  Same names, same
 *     by-reference Fortran calling convention, same array layouts and the same
 *     asynchronous-launch / blocking-collect split as the reference routine
 *     (code/mc_gpu.cu:440 and code/mc_gpu.cu:640, called from
 *     code/main_comp.f:156,193,202 and code/rad_main.f:100,102).  The reference
 *     fixes its configuration at compile time in code/param.h; here the same
 *     values are a runtime dnsmc_config, taken from dnsmc_set_default_config()
 *     or from the environment (see dnsmc_config_from_env), so a Fortran caller
 *     links this library instead of mc_gpu.o without source changes.
 *
 *  2. The handle-based dnsmc_* API: explicit configuration, table loading in
 *     the reference text formats or from raw arrays, resident fields, several
 *     snapshots per solve, band-group stratification, adaptive ray counts,
 *     integer error codes (the reference exits the process on any error,
 *     code/param.h:85-95), a status word and a bounded wait.
 *
 * Plain C types only: pointers, sizes, ints and floats.  Every function that
 * can fail returns an int error code (DNSMC_OK == 0); dnsmc_last_error()
 * gives a one-line description of the most recent failure on the calling
 * thread.
 *
 * Axis convention (the reference's): i is wall-normal (the two walls sit at
 * x = 0 and x = Lx), j and k are periodic.  Field arrays are dense, i fastest
 * (index i + imax*(j + jmax*k)) unless a function states otherwise.
 */
#ifndef DNSMC_H
#define DNSMC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes --------------------------------------------------------- */
#define DNSMC_OK            0
#define DNSMC_ERR_ARG       1   /* invalid argument or inconsistent sizes      */
#define DNSMC_ERR_STATE     2   /* call out of order (e.g. solve before tables) */
#define DNSMC_ERR_CUDA      3   /* CUDA runtime failure                         */
#define DNSMC_ERR_IO        4   /* table file missing or malformed              */
#define DNSMC_ERR_TIMEOUT   5   /* bounded wait expired; work still in flight   */
#define DNSMC_ERR_NOMEM     6   /* host or device allocation failed             */
#define DNSMC_ERR_TABLE     7   /* table values unusable (non-positive, NaN)    */
#define DNSMC_ERR_NODEVICE  8   /* no CUDA device visible                       */

/* ---- status bits (dnsmc_status) ------------------------------------------ */
#define DNSMC_STATUS_STEP_CAP   0x1u  /* a ray stopped at the per-ray step cap   */
#define DNSMC_STATUS_NONFINITE  0x2u  /* a non-finite ray contribution was seen  */
#define DNSMC_STATUS_BAD_FIELD  0x4u  /* a temperature <= 0 or NaN was supplied  */
#define DNSMC_STATUS_COPY_TIMEOUT 0x8u /* a bounded wait for an on-chip table copy
                                          ran out; the solve reports an error  */

/* ---- spectral models (reference code/param.h:48-49, `grey`) -------------- */
#define DNSMC_MODEL_CK         0  /* narrow-band correlated-k gas tables        */
#define DNSMC_MODEL_GREY_BANDS 1  /* reference grey tables: 1000 equal bands     */
#define DNSMC_MODEL_PARTICLE   2  /* reference particle-absorption tables        */
#define DNSMC_MODEL_GREY       3  /* grey medium, constant kappa, sigma*T^4      */
#define DNSMC_MODEL_TABLE      4  /* raw k(band, g, T, x_H2O) table (set_table)  */

/* ---- ray samplers ----------------------------------------------------------
 * IID: every ray draws (phi, cos theta, spectral index, alias threshold) from
 *   its own Philox4x32-10 counter; sigma from the per-ray sample variance.
 * RQMC: the rays of one (packet, band group) are nvar replicates of a Sobol'
 *   net in those four dimensions, each replicate digitally shifted by a Philox
 *   word (unbiased; the reference itself draws directions from Sobol',
 *   code/mc_gpu.cu:80-81,121); sigma from the nvar replicate means, like the
 *   reference's nVar batches (code/mc_gpu.cu:217-222).                       */
#define DNSMC_SAMPLER_IID      0
#define DNSMC_SAMPLER_RQMC     1

/* ---- field layouts -------------------------------------------------------- */
#define DNSMC_LAYOUT_DENSE     0  /* imax*jmax*kmax, i fastest, no ghosts        */
#define DNSMC_LAYOUT_FORTRAN   1  /* (imax+2)(jmax+2)(kmax+2), i fastest, ghost  */
                                  /* layer included: the reference TMC array     */

typedef struct dnsmc_config {
    /* geometry (code/param.h:4-11) */
    int   imax, jmax, kmax;      /* cells; i wall-normal, j and k periodic      */
    int   p_row;                 /* number of j-slabs (decomp_2d p_row)         */
    float Lx, Ly, Lz;            /* domain lengths [m]                           */
    int   stretched_x;           /* 1: the reference wall-normal stretching     */
                                 /* (code/definitions.h:108-134), 0: uniform    */
    /* rays (code/param.h:13-14) */
    int   nvar;                  /* batches per cell (sigma normaliser, :221)    */
    int   photmax;               /* rays per batch; rays/cell = nvar*photmax    */
    /* walls (code/param.h:56-83): west = x 0, east = x Lx; j,k periodic */
    float T_west, T_east;        /* wall temperatures [K]                        */
    float eps_west, eps_east;    /* wall emissivity, 1 = black (bdw=bde=2)      */
    /* march (code/param.h:72, :25-37) */
    float toll;                  /* transmissivity cut-off                      */
    int   max_steps;             /* per-ray step cap, 1 .. 4194304               */
    int   grid_num;              /* multigrid levels (code/param.h:18-37): rays  */
                                 /* march mg_steps steps on each grid, then    */
                                 /* continue on the next grid, 2x coarser per  */
                                 /* axis (spline-coarsened T); 1 = fine only   */
    /* spectral model */
    int   model;                 /* DNSMC_MODEL_*                                */
    float kappa;                 /* grey absorption coefficient [1/m] (GREY)     */
    int   n_groups;              /* band groups for stratified sampling (>=1)    */
    /* randomness */
    uint64_t seed;
    int   sampler;               /* DNSMC_SAMPLER_*                              */
    int   local_sampling;        /* 1: draw the spectral sample from the emission */
                                 /* spectrum at the packet's own temperature     */
                                 /* (per-temperature-bin alias tables); 0: at    */
                                 /* Tmax for every cell, as code/mc_gpu.cu:142   */
    int   control_variate;       /* 1: tally X - beta*Y with Y the same ray   */
                                 /* through the plane-averaged T and x_H2O     */
                                 /* profile; E[Y] from a 1-D layered-slab     */
                                 /* quadrature is added back (unbiased)        */
    int   cv_moments;            /* 1: also tally per-ray moments of X and the  */
                                 /* two control variates (network training)    */
    /* kernel shape (0 = automatic) */
    int   block_threads;         /* 128 or 256                                   */
    int   tile_a;                /* cells of a packet along j: 8, 16 or 32;     */
                                 /* automatic: 8 (8 x 8 packets) on the fine    */
                                 /* grid when k has 8 cells or more, else 16   */
                                 /* or 32; the widest row with grid_num > 1     */
    /* multigrid */
    int   mg_steps;              /* steps per grid before the next coarser one  */
                                 /* (the reference's maxs, 5); the last grid    */
                                 /* marches up to max_steps                     */
} dnsmc_config;

/* Raw spectral table for DNSMC_MODEL_TABLE (and the internal representation of
 * every tabulated model).  k is an absorption coefficient in 1/m on a uniform
 * T grid and a uniform x_H2O grid; it is interpolated linearly in T and x.     */
typedef struct dnsmc_table_desc {
    int   nbands, nq, nT, nX;    /* nX == 1: no x_H2O dependence                */
    float T0, dT;                /* T grid: T0 + t*dT, t = 0..nT-1              */
    float X0, dX;                /* x grid: X0 + u*dX, u = 0..nX-1              */
    const float *k;              /* [nbands][nq][nT][nX]                        */
    const float *wvc;            /* [nbands] band-centre wavenumber [1/cm]      */
    const float *dnu;            /* [nbands] band width [1/cm]                  */
    const float *wq;             /* [nq] quadrature weights (sum 1)             */
    const float *Ib;             /* [nbands][nT] band Planck intensity, or NULL */
                                 /* (then computed at wvc, code/memory_copy.cu:291) */
    /* Reference sampling data (optional).  When prob != NULL the band and
     * g-point are drawn from these CDFs at the table temperature nearest to
     * Tmax and weighted with the Planck-mean kP, as code/mc_gpu.cu:142-169 and
     * :830-896 do; otherwise the sampling density is built from k, Ib, dnu, wq
     * at Tmax (and the field-mean x_H2O).                                      */
    const float *prob;           /* [nT][nbands] band CDF                       */
    const float *probg;          /* [nT][nbands][nq] g-point CDF, or NULL       */
    const float *kP;             /* [nT] Planck-mean absorption coefficient     */
} dnsmc_table_desc;

typedef struct dnsmc_solver dnsmc_solver;

/* ---- configuration -------------------------------------------------------- */
/* The reference's shipped code/param.h values (64^3, particle tables, black
 * x-walls at 500 K, Lx=Ly=Lz=1, nVar=3, photmax=20000), except grid_num = 1:
 * rays march on the fine grid only (grid_num = 5 with mg_steps = 5 is the
 * reference's shipped multigrid; it needs the reference tables or the grey
 * model, no control variate, black walls and no particles).                 */
void dnsmc_set_default_config(dnsmc_config *cfg);
/* Overlay DNSMC_* environment variables (DNSMC_IMAX, DNSMC_JMAX, DNSMC_KMAX,
 * DNSMC_PROW, DNSMC_LX, DNSMC_LY, DNSMC_LZ, DNSMC_NVAR, DNSMC_PHOTMAX,
 * DNSMC_TWEST, DNSMC_TEAST, DNSMC_MODEL, DNSMC_GRID_NUM, DNSMC_SEED,
 * DNSMC_STRETCHED) on cfg.  Returns DNSMC_ERR_ARG on an unparsable value.     */
int  dnsmc_config_from_env(dnsmc_config *cfg);
const char *dnsmc_last_error(void);
const char *dnsmc_version(void);

/* ---- solver lifetime ------------------------------------------------------ */
int  dnsmc_create(const dnsmc_config *cfg, dnsmc_solver **out);
int  dnsmc_destroy(dnsmc_solver *s);

/* ---- tables (host-side parse; no GPU needed) ------------------------------ */
/* Read the reference text tables from dir (the reference hard-codes
 * ../distr/tables/, code/read_tables.cpp:25,43,65) for model CK (planck-mean.txt,
 * NarrBand%d.txt, prob_new2.txt; code/read_tables.cpp:20-92) or PARTICLE
 * (particles/{planck-mean,NarrBand%d,prob}.txt; code/read_tables.cpp:185-241).
 * nT, nB, nQ as in code/NarrowBand.h (52,119,16 for CK; 52,119,1 for PARTICLE).*/
int  dnsmc_load_tables_ref(dnsmc_solver *s, const char *dir, int model,
                           int nT, int nB, int nQ);
/* Reference grey tables (code/grey_tables.cpp:19-109): nB equal bands up to
 * wvmax [1/cm], kappa everywhere, T grid from 0.9*Tmin to 1.1*Tmax.  The T grid
 * depends on Tmax, so the table is rebuilt at every solve.                     */
int  dnsmc_use_grey_band_tables(dnsmc_solver *s, int nB, int nT, float wvmax,
                                float Tmin);
int  dnsmc_set_table(dnsmc_solver *s, const dnsmc_table_desc *t);
/* Binary table file (no counterpart in the reference, which parses its text
 * tables at every call, code/read_tables.cpp, as distr/write_tables.cpp:23-107
 * wrote them, and has no x_H2O axis): the solver's current table -- k(band, g,
 * T, x_H2O), band centres and widths, g weights, and the optional band Ib and
 * reference CDFs -- in one little-endian file with a 72-byte header (magic
 * "DNSMCKT1", version, sizes, grids, flags, payload length and its FNV-1a
 * hash) followed by float32 arrays.  dnsmc_load_table checks the header,
 * length and hash (DNSMC_ERR_IO) and then sets the table as dnsmc_set_table
 * does.  Parsed once, a table file serves every later solver.               */
int  dnsmc_save_table(const dnsmc_solver *s, const char *path);
int  dnsmc_load_table(dnsmc_solver *s, const char *path);
/* Copy of the parsed table (host arrays of the sizes in the desc); any pointer
 * may be NULL.  For tests of the parsers.                                      */
int  dnsmc_get_table_info(const dnsmc_solver *s, int *nbands, int *nq, int *nT,
                          int *nX, float *T0, float *dT, float *X0, float *dX);
int  dnsmc_get_table(const dnsmc_solver *s, float *k, float *wvc, float *Ib,
                     float *prob, float *probg, float *kP);

/* ---- fields and solve ------------------------------------------------------ */
/* Upload nfields snapshots of temperature [K] and optional H2O mole fraction
 * (x may be NULL: taken as 0) to device-resident storage, in the given layout.
 * Host arrays may be reused as soon as the call returns.                       */
int  dnsmc_set_fields(dnsmc_solver *s, int nfields, const float *T,
                      const float *x, int layout);
/* Same, from device pointers (dense layout), stream-ordered on the solver's
 * stream; no host copy.                                                        */
int  dnsmc_set_fields_device(dnsmc_solver *s, int nfields, const float *dT,
                             const float *dx);
/* Particles (the general medium; no counterpart in the reference's GPU path,
 * which has neither scattering, code/param.h:71, nor grey walls,
 * code/param.h:77): per band the absorption and scattering coefficients per
 * unit particle volume fraction [1/m] (nbands = the k table's bands, 1 for the
 * grey model) and the Henyey-Greenstein asymmetry g in (-1, 1).  A cell with
 * volume fraction fv absorbs k_gas + fv a_band and scatters fv s_band; the
 * particles emit at the cell temperature.  Scattering is tracked by weighted
 * delta tracking (majorant max(fv) s_band).  Both arrays NULL removes the
 * particles.  Requires MODEL_GREY or MODEL_TABLE; set the k table first.   */
int  dnsmc_set_particles(dnsmc_solver *s, int nbands, const float *absorption,
                         const float *scattering, float hg_g);
/* Volume fraction of every resident snapshot (host, the layout of
 * dnsmc_set_fields); after dnsmc_set_fields, again after every new fields.  */
int  dnsmc_set_particle_field(dnsmc_solver *s, const float *fv, int layout);
/* Cells to compute: i in [i0,i1), j in [j0,j1), k in [k0,k1) (0-based); the
 * march always sees the whole field.  Default: all cells.                      */
int  dnsmc_set_region(dnsmc_solver *s, int i0, int i1, int j0, int j1, int k0,
                      int k1);
/* Rays per cell per band group.  rays_per_packet (length = number of packets,
 * see dnsmc_packet_count) overrides it per packet when non-NULL.            */
int  dnsmc_set_rays(dnsmc_solver *s, int rays_per_group,
                    const int *rays_per_packet);
/* Ray counts per (band group, packet): rays[g * npackets + p], n_groups = the
 * band groups of the solve.  Each count >= 0 (a multiple of nvar under RQMC);
 * 0 leaves that group of the packet unsampled (its mean and variance are 0).
 * Replaced by dnsmc_set_rays / dnsmc_set_region.  No counterpart in the
 * reference, whose rays per cell are the compile-time photmax
 * (code/param.h:64).                                                         */
int  dnsmc_set_rays_per_item(dnsmc_solver *s, int n_groups, const int *rays);
/* Rays per packet proportional to local optical thickness: for every packet
 * the mean over its cells (and the resident snapshots) of
 * tau = kP(T, x_H2O) (dx dy dz)^(1/3), kP the Planck-mean absorption
 * coefficient of the tables (kappa for the grey model), gives
 * n = clamp(round(rays_per_tau * tau), min_rays, max_rays) rays per cell and
 * band group, in multiples of nvar under RQMC.  Computed on the device on
 * the solver's stream from the resident fields; replaced by dnsmc_set_rays,
 * dnsmc_set_rays_per_item or dnsmc_set_region.  No counterpart in the
 * reference (photmax rays for every cell, code/param.h:64).                 */
int  dnsmc_set_rays_adaptive(dnsmc_solver *s, float rays_per_tau, int min_rays,
                             int max_rays);
/* The per-item ray table in effect (set by dnsmc_set_rays_per_item or by a
 * control-variate network, dnsmc_cvnet_apply, or dnsmc_set_rays_adaptive):
 * *n_groups = 0 when rays are uniform, -1 for one row of per-packet counts
 * shared by all band groups, else the rows of the per-(group, packet) table;
 * rays (may be NULL) receives max(1, *n_groups) * npackets counts.          */
int  dnsmc_get_rays_per_item(dnsmc_solver *s, int *n_groups, int *rays);
int  dnsmc_packet_count(const dnsmc_solver *s, int *npackets);
/* Packet shape of the next solve: tile_a cells along j by tile_b along k.  A
 * packet is 64 cells (two per lane of a warp) on the fine grid, 32 cells
 * with grid_num > 1; the packet count and per-packet ray tables follow it.
 * No reference counterpart (the reference runs one thread per cell).        */
int  dnsmc_packet_shape(const dnsmc_solver *s, int *tile_a, int *tile_b);
/* Enqueue a solve of every resident snapshot on the solver's stream and return.*/
int  dnsmc_solve_async(dnsmc_solver *s);
/* Wait for the last solve, at most timeout_s seconds (<=0: no limit).          */
int  dnsmc_wait(dnsmc_solver *s, double timeout_s);
/* Results of the last solve, blocking: per cell of the region (dense, i fastest,
 * snapshot slowest) the radiative source Q [W/m^3] (emission minus absorption)
 * and the standard error of Q.  Either pointer may be NULL.                    */
int  dnsmc_get_results(dnsmc_solver *s, double *Q, double *sigma);
/* Host result type of the next solves.  DNSMC_RESULT_F64 (default): Q and
 * sigma cross to the host as doubles (16 bytes per cell), read with
 * dnsmc_get_results.  DNSMC_RESULT_F32: the finalize kernel rounds Q and
 * sigma to float on the device and only those cross (8 bytes per cell), read
 * with dnsmc_get_results_float (the reference returns real(4) arrays,
 * code/mc_gpu.cu:762-776; the drop-in pair uses this type).  No counterpart
 * in the reference, which copies float solution and variance back and takes
 * the square root on the host.                                              */
#define DNSMC_RESULT_F64 0
#define DNSMC_RESULT_F32 1
int  dnsmc_set_result_type(dnsmc_solver *s, int type);
/* Results of the last solve as floats, blocking (either pointer may be
 * NULL); after a DNSMC_RESULT_F64 solve the doubles are rounded here.
 * dnsmc_get_results fails with DNSMC_ERR_STATE after a DNSMC_RESULT_F32
 * solve.                                                                    */
int  dnsmc_get_results_float(dnsmc_solver *s, float *Q, float *sigma);
/* Per band group: mean and variance of the mean, [field][group][cell].         */
int  dnsmc_get_group_results(dnsmc_solver *s, double *Qg, double *varg);
/* Spline-coarsened temperature of multigrid level 1..grid_num-1 of resident
 * snapshot `field`: (imax>>level)*(jmax>>level)*(kmax>>level) values, dense,
 * i fastest (the reference's interp3D, code/spline.cpp:35-116).             */
int  dnsmc_get_coarse_field(dnsmc_solver *s, int field, int level, float *T);
/* CUDA graph replay of the solve: when enabled, the kernel sequence of a
 * solve (table coordinates, control-variate preparation, the persistent
 * march, finalize and the result copy) is captured once into a CUDA graph
 * and replayed by later solves whose launch parameters are unchanged (same
 * grid, region, ray layout, tables and buffers; the field values, ray counts
 * and coefficients in device memory may change).  A change of any of them
 * captures again.  The march timing of dnsmc_get_timing then covers the whole
 * replayed sequence.                                                        */
int  dnsmc_set_graph(dnsmc_solver *s, int enable);
/* Number of graph captures and replays so far.                              */
int  dnsmc_get_graph_info(const dnsmc_solver *s, long long *captures,
                          long long *launches);
/* Kernels this library has launched in this process, all solvers and
 * networks together (a CUDA-graph replay counts the kernel nodes of its
 * graph).  The difference across a region of code is the number of this
 * library's kernels that region launched.                                   */
int  dnsmc_get_launch_count(long long *n);
/* The solver's CUDA stream (cudaStream_t; created on first use): every solve,
 * upload and network evaluation of this solver is ordered on it, so a caller
 * can order its own work (or CUDA events) against them.                      */
int  dnsmc_get_stream(dnsmc_solver *s, void **stream);
/* Bits DNSMC_STATUS_* accumulated by the last solve.                           */
int  dnsmc_status(dnsmc_solver *s, uint32_t *status);
/* Counters of the last solve: emitted rays and ray-voxel steps (all lanes),
 * device time of the march kernel in milliseconds.                             */
int  dnsmc_get_counters(dnsmc_solver *s, double *rays, double *steps,
                        double *march_ms);
/* Ray-voxel steps of the last solve per work item (field, band group,
 * packet), summed over the item's rays: steps[(f * n_groups + g) * npackets
 * + p].  The cost model of ray allocation.                                   */
int  dnsmc_get_item_steps(dnsmc_solver *s, double *steps);
/* Device time of the last solve measured with CUDA events on the solver's
 * stream: from the first enqueued operation (sampling upload) to the end of
 * the result copy into pinned host memory, and of the march kernel alone.    */
int  dnsmc_get_timing(dnsmc_solver *s, double *solve_ms, double *march_ms);
/* Tmax used for sampling (max over fields and wall temperatures).              */
int  dnsmc_get_tmax(const dnsmc_solver *s, float *tmax);

/* ---- spectral sampling tables (for the host replay in the tests) ----------- */
/* Entries of every (temperature bin, band group): alias threshold, alias
 * index, band, g-point, weight factor W (ray weight = W * k(T_i) * Ib(T_i)).
 * Valid after a solve or dnsmc_prepare_sampling.  group_start has
 * n_tbins*n_groups+1 entries (bin major); n_tbins is 1 without local sampling.*/
int  dnsmc_get_sampling(const dnsmc_solver *s, int *n_groups, int *n_tbins,
                        int *group_start, int *n_entries, float *prob,
                        int *alias, int *band, int *gq, float *W, float *ibw);
/* Build the sampling tables for a given Tmax and mean x_H2O on the host
 * without solving (no GPU needed); dnsmc_get_sampling then returns them.     */
int  dnsmc_prepare_sampling(dnsmc_solver *s, float Tmax, float xmean);
/* The control variate has two terms: Y_a, the ray's contribution in the
 * medium of plane-averaged T and x_H2O, and Y_b, the part of Y_a from the
 * emitting plane itself.  The march tallies X - beta_a Y_a - beta_b Y_b and
 * beta_a E[Y_a] + beta_b E[Y_b] is added back.  Coefficients per (field,
 * band group, cell of the region), dense i fastest, pairs (beta_a, beta_b);
 * NULL restores (1, -1).  Any finite pair keeps the estimate unbiased.       */
int  dnsmc_set_cv_beta(dnsmc_solver *s, const float *beta);
/* The coefficients in effect (set by dnsmc_set_cv_beta or by a network,
 * dnsmc_cvnet_apply), same layout; DNSMC_ERR_STATE when none are set.       */
int  dnsmc_get_cv_beta(dnsmc_solver *s, float *beta);
/* Control-variate data of the last solve (any pointer may be NULL): layer
 * means (T_bar, x_bar) [f][imax][2], surrogate medium (k_bar, Ib_bar)
 * [f][sample][imax][2] (sample = band*nq + g), (Jhat, Ahat) [f][sample][imax][2]
 * (the exact direction means of the tabulated surrogate's collected
 * intensity and own-plane absorptance) and (E[Y_a], E[Y_b])
 * [f][group][cell][2] dense i fastest.                                      */
int  dnsmc_get_cv_data(dnsmc_solver *s, int *n_samples, float *layer, float *sur,
                       double *Jhat, double *muY);
/* The tabulated surrogate of the last control-variate solve,
 * [f][sample][imax][2][DNSMC_CV_BINS][4]: for a ray leaving the centre of
 * plane i towards the west (0) or east (1) wall with sqrt(|mu|) = (m + r) /
 * DNSMC_CV_BINS, r in [0, 1), the march reads (J0, dJ, A0, dA) of bin m and
 * takes J = J0 + r dJ (collected intensity), A = A0 + r dA (own-plane
 * absorptance).  Holds n_samples * imax * 2 * DNSMC_CV_BINS * 4 floats per field. */
#define DNSMC_CV_BINS 64
int  dnsmc_get_cv_table(dnsmc_solver *s, float *tab);
/* Per-ray moments of the last solve with cv_moments = 1, [f][group][cell][9]
 * dense i fastest: sums of X, Y_a, Y_b, X^2, Y_a^2, Y_b^2, X Y_a, X Y_b,
 * Y_a Y_b over the cell's rays (X is the plain OERM ray contribution).       */
int  dnsmc_get_cv_moments(dnsmc_solver *s, double *moments);
/* Wall-normal faces (imax+1) and periodic cell sizes used by the march.       */
int  dnsmc_get_geometry(const dnsmc_solver *s, float *xu, float *dy, float *dz);

/* ---- trace of one packet-ray (bit-exact replay tests) ---------------------- */
/* Record the voxel walk of ray r of packet p in band group g of field f: per
 * step the wall-normal index, the j/k offsets, the crossed axis, the segment
 * length and lane 0's transmissivity.  Up to max_steps records of 6 words.    */
int  dnsmc_trace_ray(dnsmc_solver *s, int f, int g, int p, int r, int max_steps,
                     int32_t *rec, int *n_steps, uint32_t *rng4);

/* ---- learned control variate ----------------------------------------------
 * No counterpart in the reference (its estimator has no control variate).
 * A small MLP (67 features -> 3 x 128 GELU -> 64 outputs; BF16 weights and
 * activations, FP32 accumulation on the tensor cores) predicts per cell and
 * band group (up to 16 groups):
 *   - the control-variate coefficients (beta_a, beta_b), as offsets from
 *     (1, -1); any finite pair keeps the estimate unbiased, the network aims
 *     at the pair of least variance;
 *   - the log of the estimator variance per ray and of the ray-voxel steps
 *     per ray, from which ray counts per (band group, packet) follow as
 *     n ~ sqrt(v / c) at the expected step cost of uniform rays.
 * Features: T, x_H2O and the signed wall-normal position 2 eta - 1 of the
 * cell, and T, x_H2O at 32 points of the wall-normal line through the cell
 * (layers ((2q+1) imax) / 64), as (T - T_center) / T_scale and
 * (x - x_center) / x_scale, rounded to bf16.
 * Training data come from solves with control_variate and cv_moments set: per
 * (cell, group) the per-ray covariances of (X, Y_a, Y_b), the estimator
 * variance and the packet's steps per ray; losses: the residual variance
 * (plus ridge * (Var Y_a dbeta_a^2 + Var Y_b dbeta_b^2)) and, for the two log
 * heads, v e^-o + o (minimised at o = log E[v]).  Adam on FP32 master weights.
 * The network lives on the device current at dnsmc_cvnet_create.            */
typedef struct dnsmc_cvnet dnsmc_cvnet;
typedef struct {
    int      n_groups;             /* band-group slots, 1..16                   */
    float    T_center, T_scale;    /* feature map of T [K]                      */
    float    x_center, x_scale;    /* feature map of x_H2O                      */
    float    lr, adam_beta1, adam_beta2, adam_eps;
    float    ridge;                /* pull of the coefficients towards (1, -1)  */
    int      batch;                /* rows per training step, multiple of 128   */
    uint64_t seed;                 /* initial weights and row shuffling         */
} dnsmc_cvnet_config;
#define DNSMC_CVNET_NFEAT  67
#define DNSMC_CVNET_NOUT   64
#define DNSMC_CVNET_NLABEL 8       /* Cxx Caa Cbb Cxa Cxb Cab v c per (cell, group) */
#define DNSMC_CVNET_BETA   1       /* dnsmc_cvnet_apply: coefficients           */
#define DNSMC_CVNET_RAYS   2       /* dnsmc_cvnet_apply: ray allocation         */
void dnsmc_cvnet_default_config(dnsmc_cvnet_config *cfg);
int  dnsmc_cvnet_create(const dnsmc_cvnet_config *cfg, dnsmc_cvnet **out);
int  dnsmc_cvnet_destroy(dnsmc_cvnet *net);
long long dnsmc_cvnet_param_count(void);
/* FP32 parameters, flat: W1[128][80] b1 W2[128][128] b2 W3[128][128] b3
 * W4[64][128] b4 (columns 67..79 of W1 are padding and stay 0); scales =
 * (S_beta, S_v, S_c), the label scales of the losses.  Either may be NULL.
 * set_params resets the Adam state.                                         */
int  dnsmc_cvnet_get_params(dnsmc_cvnet *net, float *params, float *scales);
int  dnsmc_cvnet_set_params(dnsmc_cvnet *net, const float *params,
                            const float *scales);
int  dnsmc_cvnet_save(dnsmc_cvnet *net, const char *path);
int  dnsmc_cvnet_load(const char *path, dnsmc_cvnet **out);
/* Features of every cell of the solver's region (tally order: i slowest, then
 * k, j fastest; field slowest), [rows][67] floats (the bf16 values).        */
int  dnsmc_cvnet_features(dnsmc_cvnet *net, dnsmc_solver *s, float *features);
/* Append the region's cells of the solver's last solve (control_variate and
 * cv_moments set, same region) to the network's device-resident data.  The
 * first call fixes the label scales.                                        */
int  dnsmc_cvnet_add_training_data(dnsmc_cvnet *net, dnsmc_solver *s);
int  dnsmc_cvnet_clear_training_data(dnsmc_cvnet *net);
long long dnsmc_cvnet_training_rows(const dnsmc_cvnet *net);
/* Adam over the data for `epochs` shuffled passes; loss[4] (may be NULL)
 * receives the mean losses of the last pass: total, beta, variance, cost.   */
int  dnsmc_cvnet_train(dnsmc_cvnet *net, int epochs, double *loss);
/* Forward pass on host features [rows][67] -> out [rows][64].               */
int  dnsmc_cvnet_eval(dnsmc_cvnet *net, const float *features, long long rows,
                      float *out);
/* One forward + backward pass without update on host features and labels
 * [rows][n_groups][8]: grad receives dnsmc_cvnet_param_count() floats of
 * d(mean loss)/d(params), loss[4] as dnsmc_cvnet_train.                     */
int  dnsmc_cvnet_gradient(dnsmc_cvnet *net, const float *features,
                          const float *labels, int n_groups, long long rows,
                          float *grad, double *loss);
/* Evaluate the network on the solver's resident fields and region and set,
 * on the solver's stream, the control-variate coefficients (flags & BETA)
 * and/or the per-(group, packet) ray counts (flags & RAYS) of its next
 * solves: n = clamp(round(lambda sqrt(v/c)), min_rays, max_rays) in multiples
 * of nvar (RQMC), lambda such that the expected steps equal those of
 * mean_rays uniform rays.  Requires max(2, nvar) <= min_rays <= mean_rays
 * <= max_rays.  dnsmc_set_rays / dnsmc_set_cv_beta(NULL) undo it.           */
int  dnsmc_cvnet_apply(dnsmc_cvnet *net, dnsmc_solver *s, int flags,
                       int mean_rays, int min_rays, int max_rays);

/* ---- allocation-free grey solve -------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory while they run: host codes whose pool allocator owns all free device
 * memory from start-up, or runs that must keep a fixed memory footprint after
 * initialisation.  It solves a grey medium (cfg->model == DNSMC_MODEL_GREY,
 * IID sampler, nvar*photmax rays per cell, the whole grid) and calls no
 * cudaMalloc/cudaFree or allocating library routine: its intermediate buffers
 * live in one fixed file-scope device array of about 5.3 MB that every GPU
 * loading the library holds until the process exits.
 *   xu   : host, imax+1 wall-normal face coordinates [m] (e.g. from
 *          dnsmc_get_geometry or the caller's own grid), copied to the
 *          device at every call, in stream order
 *   dT   : device, imax*jmax*kmax temperatures [K], dense, i fastest
 *   dQ   : device, imax*jmax*kmax doubles out: Q [W/m^3], dense, i fastest
 *   dvar : device, imax*jmax*kmax doubles out: variance of Q
 *   dstatus: device, one uint32 out, or NULL: the DNSMC_STATUS_* bits of
 *          this solve (DNSMC_STATUS_BAD_FIELD for a temperature <= 0 or
 *          NaN, DNSMC_STATUS_STEP_CAP, DNSMC_STATUS_NONFINITE), written on
 *          the stream after Q and var; read it once the stream has finished.
 *          Q and var are not to be used when it is non-zero.
 *   stream: CUDA stream (NULL: default stream); the call only enqueues.
 * Limits: at most DNSMC_NOALLOC_MAX_CELLS cells and imax <= DNSMC_NOALLOC_MAX_IMAX;
 * larger grids return DNSMC_ERR_ARG, as does max_steps outside
 * [1, 4194304] (the handle API's bound).  The first call on a device looks
 * up the device address of the array (cudaGetSymbolAddress) with that device
 * current; make that first call before any stream capture.  All calls share
 * the one array and it keeps the previous call's contents (each call clears
 * what must start at zero); calls whose work overlaps on the GPU (different
 * streams, or host threads, without ordering between them) race on it.     */
#define DNSMC_NOALLOC_MAX_CELLS 262144   /* 64^3 */
#define DNSMC_NOALLOC_MAX_IMAX  1024
int  dnsmc_solve_grey_noalloc(const dnsmc_config *cfg, const float *xu,
                              const float *dT, double *dQ, double *dvar,
                              uint32_t *dstatus, void *stream);

/* ---- correlated-k tables from line-by-line spectra -------------------------
 * The reference's offline table generator (distr/correlatedK.cpp:145-300,
 * correlatedKT, and the band means of distr/calc_prob.cpp:17-119) on the GPU,
 * for every temperature, H2O mole fraction and narrow band at once: per band
 * the k-distribution of the spectrum (n_pwrk bins uniform in k^0.1 between
 * the band's smallest and largest k, each interval between neighbouring
 * points at its midpoint k, weighted by its share dwv / (wv_right - wv_left)
 * of the band), its cumulative g-function, and k at the quadrature points gq
 * by linear interpolation in g.  The spectra are uniform in wavenumber
 * (spacing dwv, as the reference's 0.01 1/cm); band b holds the points
 * [first[b], first[b] + count[b]).  The output k has the layout of
 * dnsmc_table_desc.k ([nbands][nq][nT][nX]), so it feeds dnsmc_set_table
 * (with the band centres, widths and the quadrature weights) directly.    */
typedef struct dnsmc_lbl_desc {
    int nT, nX;                  /* spectra: temperatures x mole fractions       */
    long long npts;              /* points of every spectrum                     */
    double wv0, dwv;             /* wavenumber of point 0 and spacing [1/cm]     */
    const double *kappa;         /* [nT][nX][npts] absorption coefficient [1/m]  */
    int nbands;
    const long long *first;      /* [nbands] first point of each band            */
    const int *count;            /* [nbands] points of each band (>= 2)          */
    const double *wv_left;       /* [nbands] band edges [1/cm]                   */
    const double *wv_right;
    int nq;
    const double *gq;            /* [nq] quadrature points, ascending in (0, 1)  */
    int n_pwrk;                  /* bins of the k-distribution, 2 .. 50000       */
                                 /* (the reference's 10000)                     */
} dnsmc_lbl_desc;
/* kq: [nbands][nq][nT][nX] floats out; kavg: [nT][nX][nbands] band-mean k out
 * (calc_prob.cpp's k_avg), or NULL.  A band whose k is constant gets that k
 * at every g (the reference divides by a zero bin width there).  Blocking;
 * allocates and frees its own device buffers.                                */
int  dnsmc_ck_from_lbl(const dnsmc_lbl_desc *d, float *kq, double *kavg);

/* ---- reference drop-in (code/mc_gpu.cu:440, :640) -------------------------- */
/* Tfort: real(4) TMC(0:imax+1,0:jmax+1,0:kmax+1), i fastest, whole domain with
 * ghost layers.  *ystart: 1-based global j of this rank's slab (xstart(2)).
 * Enqueues the solve of the slab's cells and returns (the caller runs DNS
 * steps meanwhile).  On error prints to stderr and exits, as the reference.   */
void mc_gpu_(float *Tfort, int *ystart);
/* resfort, varfort: real(4) (0:imax+1, 0:jmax/p_row+1, 0:kmax+1), i fastest.
 * Blocks, then writes Q [W/m^3] and its standard deviation with the
 * reference's 1/((nVar-0.5)(nVar-1)) normaliser into interior cells only.     */
void get_results_(float *resfort, float *varfort);
/* Configure the instance the drop-in pair uses (optional; otherwise the
 * defaults overlaid with the environment are used on the first mc_gpu_ call).
 * table_dir NULL means "../distr/tables" as the reference.                    */
int  dnsmc_dropin_configure(const dnsmc_config *cfg, const char *table_dir);
int  dnsmc_dropin_release(void);

#ifdef __cplusplus
}
#endif
#endif /* DNSMC_H */
