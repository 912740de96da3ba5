// mc_host.cpp -- host runtime behind the C ABI of include/dnsmc.h.
//
// Replaces the reference host path (code/mc_gpu.cu:440-784, code/memory_copy.cu,
// code/read_tables.cpp, code/grey_tables.cpp): the reference rebuilds every
// device object per call and ends with cudaDeviceReset; here tables, fields
// and buffers are persistent per solver, the solve is one stream-ordered
// sequence (sampling upload, march, finalize, device-to-host copy), and every
// failure is an error code instead of exit(1).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/dnsmc.h"
#include "mc_internal.h"

using namespace dnsmc;

namespace {

thread_local std::string g_err;

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CUDA_TRY(x)                                                                       \
    do {                                                                                  \
        cudaError_t e_ = (x);                                                             \
        if (e_ != cudaSuccess)                                                            \
            return fail(DNSMC_ERR_CUDA, "%s failed: %s", #x, cudaGetErrorString(e_));     \
    } while (0)

#define TRY(x)                   \
    do {                         \
        int rc_ = (x);           \
        if (rc_ != DNSMC_OK) return rc_; \
    } while (0)

constexpr double kSigma = 5.670373e-08;  // code/param.h:70
constexpr double kPi = 3.14159265358979323846;

// Band-centre Planck intensity per unit wavenumber [W/(m^2 sr m^-1)], nu in
// 1/cm: the reference I_blackC (code/memory_copy.cu:291-300), same FP32 steps.
float planck_band(float T, float nu) {
    if (!(T > 0.0f)) return 0.0f;
    const float C1 = 3.741771790075259e-16f;
    const float C2 = 0.014387741858429f;
    const float n100 = nu * 100.0f;
    const float n3 = n100 * n100 * n100;
    const float den = expf(C2 * nu * 100.0f / T) - 1.0f;
    return (float)(1.0 / kPi * (double)C1 * (double)n3 / (double)den);
}

// 16 positive nodes and weights of 32-point Gauss-Legendre on [-1, 1]: the
// g-quadrature of code/NarrowBand.h:201-207 (computed, not tabulated).
void gauss_half(int nq, std::vector<float> &gq, std::vector<float> &wq) {
    const int n = 2 * nq;
    std::vector<double> x(n), w(n);
    for (int i = 0; i < n; ++i) {
        double z = cos(kPi * (i + 0.75) / (n + 0.5));
        for (int it = 0; it < 100; ++it) {
            double p1 = 1.0, p2 = 0.0;
            for (int j = 1; j <= n; ++j) {
                const double p3 = p2;
                p2 = p1;
                p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
            }
            const double pp = n * (z * p1 - p2) / (z * z - 1.0);
            const double z1 = z;
            z = z1 - p1 / pp;
            if (fabs(z - z1) < 1e-15) {
                x[i] = z;
                w[i] = 2.0 / ((1.0 - z * z) * pp * pp);
                break;
            }
        }
    }
    gq.clear();
    wq.clear();
    for (int i = n - 1; i >= 0; --i)
        if (x[i] > 0) { gq.push_back((float)x[i]); wq.push_back((float)w[i]); }
}

struct HostTable {
    int nbands = 0, nq = 0, nT = 0, nX = 1;
    float T0 = 0.f, dT = 1.f, X0 = 0.f, dX = 1.f;
    std::vector<float> k, wvc, dnu, wq, Ib, prob, probg, kP;
    bool ref_sampling = false;
    bool valid = false;
    // reference grey bands (rebuilt from Tmax at every solve)
    bool grey_bands = false;
    int gb_nB = 0, gb_nT = 0;
    float gb_wvmax = 0.f, gb_Tmin = 0.f, gb_kappa = 1.f;
};

// Reference wall-normal grid (code/definitions.h:108-134), FP32 like the
// reference; uniform when stretched == 0.
void make_faces(int im, float L, int stretched, std::vector<float> &xu) {
    xu.assign(im + 1, 0.0f);
    if (!stretched) {
        for (int i = 0; i <= im; ++i) xu[i] = (float)i * (L / (float)im);
        xu[im] = L;
        return;
    }
    const int im0 = im;
    std::vector<float> xu0(im0 + 1, 0.0f);
    for (int i = 1; i < im0 / 2 + 1; ++i) {
        const float r = (1.f * i) / im0;
        const float dx = (float)(0.5 - 1.45 * (r - 0.5) * (r - 0.5));
        xu0[i] = xu0[i - 1] + dx;
    }
    const float xnorm = xu0[im0 / 2];
    for (int i = 1; i < im0 / 2 + 1; ++i) xu0[i] = (float)(L / 2. * xu0[i] / xnorm);
    for (int i = im0; i > im0 / 2; --i) xu0[i] = L - xu0[im0 - i];
    for (int i = 1; i < im + 1; ++i) xu[i] = xu0[i * im0 / im];
}

// ---- multigrid: coarse grids and spline-coarsened temperature --------------
// Level l has (imax, jmax, kmax) >> l cells.  Its wall-normal faces are the
// reference grid at that resolution (code/definitions.h:68-136): every
// 2^l-th fine face when stretched, i * Lx / im when uniform; j and k faces
// are i * L / n.  The temperature of a coarse cell is the fine field
// interpolated at the coarse cell centre by separable natural cubic splines
// through the fine cell centres, x first, then y, then z (the reference's
// interp3D, code/spline.cpp:35-116, with spline/splint, :119-170).
void coarse_faces(int im0, int l, float L, int stretched, std::vector<float> &xu) {
    const int im = im0 >> l;
    xu.assign(im + 1, 0.0f);
    if (!stretched) {
        for (int i = 0; i <= im; ++i) xu[i] = (float)i * (L / (float)im);
        xu[im] = L;
        return;
    }
    std::vector<float> f;
    make_faces(im0, L, 1, f);
    for (int i = 0; i <= im; ++i) xu[i] = f[(size_t)i * im0 / im];
}

// centres c[1..n] of faces u[0..n] (1-based, as the splines below)
void centres(const std::vector<float> &u, std::vector<float> &c) {
    const int n = (int)u.size() - 1;
    c.assign(n + 2, 0.0f);
    for (int i = 1; i <= n; ++i) c[i] = (u[i - 1] + u[i]) * 0.5f;
}

void uniform_faces(int n, float L, std::vector<float> &u) {
    u.assign(n + 1, 0.0f);
    const float d = L / (float)n;
    for (int i = 0; i <= n; ++i) u[i] = (float)i * d;
}

// Sobol' direction numbers of four dimensions (Bratley-Fox recurrence on the
// primitive polynomials 1, x+1, x^2+x+1, x^3+x+1 with initial m = 1 | 1 |
// 1,3 | 1,3,1), 32 bits.
void sobol_directions(uint32_t v[4][32]) {
    const int deg[4] = {0, 1, 2, 3};
    const int poly[4] = {0, 0, 1, 1};  // interior coefficients a_1..a_{s-1}
    const uint32_t init[4][3] = {{1, 0, 0}, {1, 0, 0}, {1, 3, 0}, {1, 3, 1}};
    for (int d = 0; d < 4; ++d) {
        uint32_t m[33] = {0};
        if (deg[d] == 0) {
            for (int k = 1; k <= 32; ++k) m[k] = 1;
        } else {
            const int sd = deg[d];
            for (int k = 1; k <= sd; ++k) m[k] = init[d][k - 1];
            for (int k = sd + 1; k <= 32; ++k) {
                uint32_t x = m[k - sd] ^ (m[k - sd] << sd);
                for (int i = 1; i < sd; ++i)
                    if ((poly[d] >> (sd - 1 - i)) & 1) x ^= m[k - i] << i;
                m[k] = x;
            }
        }
        for (int k = 1; k <= 32; ++k) v[d][k - 1] = m[k] << (32 - k);
    }
}

template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    int ensure(size_t want) {
        if (want <= n) return DNSMC_OK;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        if (want == 0) return DNSMC_OK;
        cudaError_t e = cudaMalloc((void **)&p, want * sizeof(T));
        if (e != cudaSuccess) return fail(DNSMC_ERR_NOMEM, "cudaMalloc(%zu bytes): %s", want * sizeof(T), cudaGetErrorString(e));
        n = want;
        return DNSMC_OK;
    }
    void release() { if (p) cudaFree(p); p = nullptr; n = 0; }
};

template <class T>
struct PinBuf {
    T *p = nullptr;
    size_t n = 0;
    int ensure(size_t want) {
        if (want <= n) return DNSMC_OK;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        if (want == 0) return DNSMC_OK;
        cudaError_t e = cudaMallocHost((void **)&p, want * sizeof(T));
        if (e != cudaSuccess) return fail(DNSMC_ERR_NOMEM, "cudaMallocHost(%zu bytes): %s", want * sizeof(T), cudaGetErrorString(e));
        n = want;
        return DNSMC_OK;
    }
    void release() { if (p) cudaFreeHost(p); p = nullptr; n = 0; }
};

}  // namespace

struct dnsmc_solver {
    dnsmc_config cfg{};
    int device = 0;
    bool dev_ready = false;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_march0 = nullptr, ev_march1 = nullptr, ev_done = nullptr, ev_solve0 = nullptr;
    bool solved = false, in_flight = false;
    int solved_result_type = 0;               // result type of the last solve

    // geometry
    std::vector<float> fw;
    float da = 0.f, db = 0.f;
    DevBuf<float> d_fw;

    // tables
    HostTable tab;
    DevBuf<float> d_k, d_ib, d_ibw;
    DevBuf<float2> d_slab;   // per spectral sample: k pairs then the band's Ib pairs
    int slab_len = 0, slab_klen = 0;
    DevBuf<int2> d_posT;   // per cell (ti, ft) for T-only tables
    DevBuf<int4> d_posTX;  // per cell (ti*(nX-1)+xi, ft, fx, ti)
    bool tables_dirty = true;

    // fields
    int nfields = 0;
    bool have_x = false;
    float tmax_fields = 0.f, tmin_fields = 0.f;
    double xsum = 0.0;
    DevBuf<float> d_fieldT;
    DevBuf<float2> d_fieldTX;
    DevBuf<float> d_raw;
    DevBuf<double> d_stat_part;
    DevBuf<double> d_stat_out;

    // region and rays
    int r_i0 = 0, r_i1 = 0, r_j0 = 0, r_j1 = 0, r_k0 = 0, r_k1 = 0;
    int rays = 0;
    std::vector<int> rays_pp;                // [group][packet] when rays_pg > 0, else [packet]
    int rays_pg = 0;                         // band groups of a per-item ray table (0: per packet)
    bool rays_dev = false;                   // d_rays_pp was written on the device (no host copy)
    int rays_np = 0;                         // packets the per-packet / per-item rays were set for
    DevBuf<int> d_rays_pp;
    DevBuf<double2> d_rays_rcp;              // (1/N, 1/(N-1)) of d_rays_pp, written by the finalize launch
    DevBuf<unsigned long long> d_item_steps; // steps per (field, group, packet) of the last solve
    DevBuf<unsigned int> d_order, d_order_hist;  // longest-first queue order (per-item ray tables)
    DevBuf<float> d_kP;                      // Planck-mean absorption coefficient on the table grid

    // multigrid: spline-coarsened temperatures of levels 1..grid_num-1
    DevBuf<float> d_mgT, d_mgfw;
    DevBuf<float> d_mgpos, d_mgtmp;          // spline positions; coarsening passes' scratch
    long long mg_off[kMaxLevels] = {0};
    int mg_fwoff[kMaxLevels] = {0};
    int mg_fields = 0;

    // particles (general medium): per-band coefficients per unit volume
    // fraction and the volume-fraction field of the resident snapshots
    std::vector<float2> part;
    float hg_g = 0.f;
    DevBuf<float2> d_part;
    DevBuf<float> d_fieldV, d_layerV;
    int fv_fields = 0;
    float fv_max = 0.f;
    double fv_mean = 0.0;

    // sampling of the last solve
    float tmax_used = 0.f;
    std::vector<SpecEntry> entries;
    std::vector<int> group_start, group_empty;
    std::vector<float> ibw;
    DevBuf<SpecEntry> d_entries;
    DevBuf<int> d_group_start, d_group_empty;
    int mode = MODE_GREY;
    int n_groups_used = 1, n_tbins_used = 1;

    // control variate
    std::vector<double> Ccoef;               // [band*nq+g] target coefficients
    std::vector<int> cv_grp, cv_sid;
    std::vector<double> cv_C;
    std::vector<float> cv_Cf;
    DevBuf<int> d_cv_grp, d_cv_sid;
    DevBuf<double> d_cv_C;
    DevBuf<float2> d_layer, d_sur;
    DevBuf<double2> d_Jhat, d_muY;
    DevBuf<double> d_cvnodes;                // node sums of E[Y] (float pairs, 8 bytes each)
    DevBuf<float4> d_Jf;
    DevBuf<float4> d_surtab;                 // tabulated surrogate [f][sample][nw][2][kSurBins]
    DevBuf<float> d_cv_Cf;
    DevBuf<float2> d_beta;
    DevBuf<double> d_moments;
    bool beta_set = false;
    int cv_samples = 0;
    // the spectral sampling tables on the device (entries, group bounds,
    // wall intensities, control-variate sample lists) and what they were
    // built from: a solve rebuilds and uploads them only when that changed
    bool sampling_valid = false, cv_uploaded = false;
    double sampling_key[8] = {};
    std::vector<float2> sampling_part;

    // outputs
    DevBuf<double2> d_tally;
    DevBuf<double> d_Q, d_var, d_sig, d_Qg, d_varg;
    PinBuf<double> h_Q, h_sig;
    // DNSMC_RESULT_F32: the finalize also writes Q and sqrt(var * sig_scale)
    // as floats and only those cross to the host (8 bytes per cell)
    int result_type = DNSMC_RESULT_F64;
    double sig_scale = 1.0;
    DevBuf<float> d_Qf, d_sigf;
    PinBuf<float> h_Qf, h_sigf;
    DevBuf<unsigned int> d_misc;  // [0] queue, [1] status
    DevBuf<unsigned long long> d_counters;
    unsigned long long h_counters[2] = {0, 0};
    unsigned int h_status = 0;
    float march_ms = 0.f, solve_ms = 0.f;
    MarchParams last{};
    FinalizeParams lastF{};
    // CUDA graph of the solve's kernel sequence (dnsmc_set_graph)
    bool graph_on = false;
    cudaGraphExec_t graph_exec = nullptr;
    std::vector<unsigned char> graph_key;
    long long graph_captures = 0, graph_launches = 0;
    long long graph_kernels = 0;             // kernel nodes of the captured graph
};

namespace {

// The device side of a solver (stream, events, faces) is created on first
// use, so table parsing and sampling construction work without a GPU.
int ensure_device(dnsmc_solver *s) {
    if (s->dev_ready) {
        CUDA_TRY(cudaSetDevice(s->device));
        return DNSMC_OK;
    }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev < 1) return fail(DNSMC_ERR_NODEVICE, "no CUDA device: %s", cudaGetErrorString(e));
    CUDA_TRY(cudaGetDevice(&s->device));
    CUDA_TRY(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreate(&s->ev_march0));
    CUDA_TRY(cudaEventCreate(&s->ev_march1));
    CUDA_TRY(cudaEventCreate(&s->ev_done));
    CUDA_TRY(cudaEventCreate(&s->ev_solve0));
    s->dev_ready = true;
    {
        uint32_t dirs[4][32];
        sobol_directions(dirs);
        const int rc = upload_sobol_dirs(dirs);
        if (rc) return fail(DNSMC_ERR_CUDA, "Sobol' table upload: %s", cudaGetErrorString((cudaError_t)rc));
    }
    if (const int rc = cv_table_allow_smem())
        return fail(DNSMC_ERR_CUDA, "table kernel shared memory: %s", cudaGetErrorString((cudaError_t)rc));
    if (int rc = s->d_fw.ensure(s->fw.size())) return rc;
    CUDA_TRY(cudaMemcpy(s->d_fw.p, s->fw.data(), s->fw.size() * sizeof(float), cudaMemcpyHostToDevice));
    return DNSMC_OK;
}

int set_device(dnsmc_solver *s) { return ensure_device(s); }

int check_config(const dnsmc_config &c) {
    if (c.imax < 1 || c.jmax < 1 || c.kmax < 1) return fail(DNSMC_ERR_ARG, "imax, jmax, kmax must be >= 1");
    if (c.p_row < 1 || c.jmax % c.p_row) return fail(DNSMC_ERR_ARG, "jmax (%d) must be a multiple of p_row (%d)", c.jmax, c.p_row);
    if (!(c.Lx > 0) || !(c.Ly > 0) || !(c.Lz > 0)) return fail(DNSMC_ERR_ARG, "Lx, Ly, Lz must be > 0");
    if (c.nvar < 1 || c.photmax < 1) return fail(DNSMC_ERR_ARG, "nvar and photmax must be >= 1");
    if (!(c.toll > 0) || c.toll >= 1) return fail(DNSMC_ERR_ARG, "toll must be in (0,1)");
    // the march counts crossings in FP32 (exact below 2^22 per axis)
    if (c.max_steps < 1 || c.max_steps > (1 << 22)) return fail(DNSMC_ERR_ARG, "max_steps must be in [1, 4194304]");
    if (c.grid_num < 1 || c.grid_num > kMaxLevels) return fail(DNSMC_ERR_ARG, "grid_num must be 1..%d", kMaxLevels);
    if (c.grid_num > 1) {
        const int r = 1 << (c.grid_num - 1);
        if (c.imax % r || c.jmax % r || c.kmax % r)
            return fail(DNSMC_ERR_ARG, "grid_num %d needs imax, jmax, kmax divisible by %d", c.grid_num, r);
        if (c.mg_steps < 1) return fail(DNSMC_ERR_ARG, "mg_steps must be >= 1");
    }
    if (c.model < 0 || c.model > 4) return fail(DNSMC_ERR_ARG, "unknown model %d", c.model);
    if (c.n_groups < 1) return fail(DNSMC_ERR_ARG, "n_groups must be >= 1");
    if (c.sampler != DNSMC_SAMPLER_IID && c.sampler != DNSMC_SAMPLER_RQMC) return fail(DNSMC_ERR_ARG, "unknown sampler %d", c.sampler);
    if (c.sampler == DNSMC_SAMPLER_RQMC && c.nvar < 2) return fail(DNSMC_ERR_ARG, "the RQMC sampler needs nvar >= 2 replicates");
    if (c.local_sampling != 0 && c.local_sampling != 1) return fail(DNSMC_ERR_ARG, "local_sampling must be 0 or 1");
    if (c.control_variate != 0 && c.control_variate != 1) return fail(DNSMC_ERR_ARG, "control_variate must be 0 or 1");
    if (c.cv_moments != 0 && c.cv_moments != 1) return fail(DNSMC_ERR_ARG, "cv_moments must be 0 or 1");
    if (c.cv_moments && !c.control_variate) return fail(DNSMC_ERR_ARG, "cv_moments needs control_variate = 1");
    // the surrogate table's sweep keeps per-plane sums of the whole wall-normal
    // line in shared memory (44 bytes a plane)
    if (c.control_variate && c.imax > kCvMaxPlanes)
        return fail(DNSMC_ERR_ARG, "the control variate supports imax <= %d", kCvMaxPlanes);
    if (c.block_threads && c.block_threads != 128 && c.block_threads != 256)
        return fail(DNSMC_ERR_ARG, "block_threads must be 0, 128 or 256");
    if (c.tile_a && c.tile_a != 8 && c.tile_a != 16 && c.tile_a != 32)
        return fail(DNSMC_ERR_ARG, "tile_a must be 0, 8, 16 or 32");
    if (!(c.eps_west > 0.0f && c.eps_west <= 1.0f) || !(c.eps_east > 0.0f && c.eps_east <= 1.0f))
        return fail(DNSMC_ERR_ARG, "wall emissivities must be in (0, 1]");
    if (!(c.T_west >= 0) || !(c.T_east >= 0)) return fail(DNSMC_ERR_ARG, "wall temperatures must be >= 0");
    return DNSMC_OK;
}

// ---- reference text-format readers ---------------------------------------
FILE *open_table(const std::string &path) { return fopen(path.c_str(), "r"); }

int read_ck_tables(const std::string &dir, int nT, int nB, int nQ, HostTable &t) {
    // planck-mean.txt: "T kP kPr kM" (code/read_tables.cpp:25-30)
    std::vector<float> Tnb(nT), kP(nT);
    FILE *fp = open_table(dir + "/planck-mean.txt");
    if (!fp) return fail(DNSMC_ERR_IO, "cannot open %s/planck-mean.txt", dir.c_str());
    for (int i = 0; i < nT; ++i) {
        float d1, d2;
        if (fscanf(fp, "%f %e %e %e", &Tnb[i], &kP[i], &d1, &d2) != 4) { fclose(fp); return fail(DNSMC_ERR_IO, "planck-mean.txt: bad row %d", i); }
    }
    fclose(fp);
    t.nbands = nB; t.nq = nQ; t.nT = nT; t.nX = 1;
    t.T0 = Tnb[0]; t.dT = Tnb[1] - Tnb[0]; t.X0 = 0.f; t.dX = 1.f;
    t.k.assign((size_t)nB * nQ * nT, 0.f);
    t.wvc.assign(nB, 0.f); t.dnu.assign(nB, 0.f);
    // NarrBand%d.txt: "wl wr wvc" then nT rows "T cuprob kavg kq[nQ]" (:339-359)
    for (int b = 0; b < nB; ++b) {
        char name[64];
        snprintf(name, sizeof name, "/NarrBand%d.txt", b);
        fp = open_table(dir + name);
        if (!fp) return fail(DNSMC_ERR_IO, "cannot open %s%s", dir.c_str(), name);
        float wl, wr;
        if (fscanf(fp, "%e %e %e", &wl, &wr, &t.wvc[b]) != 3) { fclose(fp); return fail(DNSMC_ERR_IO, "%s: bad header", name); }
        t.dnu[b] = wr - wl;
        for (int i = 0; i < nT; ++i) {
            float T, cp, kavg;
            if (fscanf(fp, "%f %f %f", &T, &cp, &kavg) != 3) { fclose(fp); return fail(DNSMC_ERR_IO, "%s: bad row %d", name, i); }
            for (int g = 0; g < nQ; ++g) {
                float v;
                if (fscanf(fp, "%e", &v) != 1) { fclose(fp); return fail(DNSMC_ERR_IO, "%s: bad row %d", name, i); }
                t.k[((size_t)b * nQ + g) * nT + i] = v;
            }
        }
        fclose(fp);
    }
    // prob_new2.txt: nT*nB rows "T nb cuprob probg[nQ]" (:364-386)
    t.prob.assign((size_t)nT * nB, 0.f);
    t.probg.assign((size_t)nT * nB * nQ, 0.f);
    fp = open_table(dir + "/prob_new2.txt");
    if (!fp) return fail(DNSMC_ERR_IO, "cannot open %s/prob_new2.txt", dir.c_str());
    for (int i = 0; i < nT; ++i)
        for (int b = 0; b < nB; ++b) {
            float T;
            int nb;
            if (fscanf(fp, "%f %d %e", &T, &nb, &t.prob[(size_t)i * nB + b]) != 3) { fclose(fp); return fail(DNSMC_ERR_IO, "prob_new2.txt: bad row"); }
            for (int g = 0; g < nQ; ++g)
                if (fscanf(fp, "%e", &t.probg[((size_t)i * nB + b) * nQ + g]) != 1) { fclose(fp); return fail(DNSMC_ERR_IO, "prob_new2.txt: bad row"); }
        }
    fclose(fp);
    t.kP = kP;
    std::vector<float> gq;
    if (nQ == 16) gauss_half(16, gq, t.wq); else t.wq.assign(nQ, 1.0f / nQ);
    t.ref_sampling = true;
    return DNSMC_OK;
}

int read_particle_tables(const std::string &dir0, int nT, int nB, HostTable &t) {
    const std::string dir = dir0 + "/particles";
    std::vector<float> Tnb(nT), kP(nT);
    FILE *fp = open_table(dir + "/planck-mean.txt");  // "T kP" (code/read_tables.cpp:491-496)
    if (!fp) return fail(DNSMC_ERR_IO, "cannot open %s/planck-mean.txt", dir.c_str());
    for (int i = 0; i < nT; ++i)
        if (fscanf(fp, "%f %e", &Tnb[i], &kP[i]) != 2) { fclose(fp); return fail(DNSMC_ERR_IO, "particles/planck-mean.txt: bad row %d", i); }
    fclose(fp);
    t.nbands = nB; t.nq = 1; t.nT = nT; t.nX = 1;
    t.T0 = Tnb[0]; t.dT = Tnb[1] - Tnb[0]; t.X0 = 0.f; t.dX = 1.f;
    t.k.assign((size_t)nB * nT, 0.f);
    t.wvc.assign(nB, 0.f); t.dnu.assign(nB, 0.f);
    for (int b = 0; b < nB; ++b) {  // "wl wr wvc kq ..." (:505-518), kq constant in T
        char name[64];
        snprintf(name, sizeof name, "/NarrBand%d.txt", b);
        fp = open_table(dir + name);
        if (!fp) return fail(DNSMC_ERR_IO, "cannot open %s%s", dir.c_str(), name);
        float wl, wr, kq;
        if (fscanf(fp, "%e %e %e %e", &wl, &wr, &t.wvc[b], &kq) != 4) { fclose(fp); return fail(DNSMC_ERR_IO, "particles%s: bad header", name); }
        fclose(fp);
        t.dnu[b] = wr - wl;
        for (int i = 0; i < nT; ++i) t.k[(size_t)b * nT + i] = kq;
    }
    t.prob.assign((size_t)nT * nB, 0.f);  // prob.txt: "T nb cuprob" (:520-540)
    fp = open_table(dir + "/prob.txt");
    if (!fp) return fail(DNSMC_ERR_IO, "cannot open %s/prob.txt", dir.c_str());
    for (int i = 0; i < nT; ++i)
        for (int b = 0; b < nB; ++b) {
            float T;
            int nb;
            if (fscanf(fp, "%f %d %e", &T, &nb, &t.prob[(size_t)i * nB + b]) != 3) { fclose(fp); return fail(DNSMC_ERR_IO, "particles/prob.txt: bad row"); }
        }
    fclose(fp);
    t.probg.clear();
    t.kP = kP;
    t.wq.assign(1, 1.0f);
    t.ref_sampling = true;
    return DNSMC_OK;
}

// Reference grey tables (code/grey_tables.cpp:19-109 / code/read_tables.cpp:404-483)
void build_grey_band_tables(HostTable &t, float Tmax) {
    const int nB = t.gb_nB, nT = t.gb_nT;
    std::vector<float> Tnb(nT);
    for (int i = 0; i < nT; ++i)
        Tnb[i] = t.gb_Tmin * 0.9f + (Tmax * 1.1f - t.gb_Tmin * 0.9f) * ((float)i) / ((float)nT);
    t.nbands = nB; t.nq = 1; t.nT = nT; t.nX = 1;
    t.T0 = Tnb[0]; t.dT = Tnb[1] - Tnb[0];
    t.X0 = 0.f; t.dX = 1.f;
    std::vector<float> wvl(nB), wvr(nB);
    wvl[0] = 0;
    for (int i = 1; i < nB; ++i) wvl[i] = wvl[i - 1] + t.gb_wvmax / nB;
    wvr[0] = t.gb_wvmax / nB;
    for (int i = 1; i < nB; ++i) wvr[i] = wvr[i - 1] + t.gb_wvmax / nB;
    t.wvc.resize(nB); t.dnu.resize(nB);
    for (int i = 0; i < nB; ++i) { t.wvc[i] = (float)((wvl[i] + wvr[i]) / 2.); t.dnu[i] = wvr[i] - wvl[i]; }
    t.k.assign((size_t)nB * nT, t.gb_kappa);
    t.kP.assign(nT, t.gb_kappa);
    t.Ib.assign((size_t)nB * nT, 0.f);
    for (int b = 0; b < nB; ++b)
        for (int i = 0; i < nT; ++i) t.Ib[(size_t)b * nT + i] = planck_band(Tnb[i], t.wvc[b]);
    t.prob.assign((size_t)nT * nB, 0.f);
    for (int i = 0; i < nT; ++i) {
        float acc = t.Ib[(size_t)0 * nT + i] * (wvr[0] - wvl[0]) * 100;
        t.prob[(size_t)i * nB] = acc;
        for (int b = 1; b < nB; ++b) {
            acc = acc + t.Ib[(size_t)b * nT + i] * (wvr[b] - wvl[b]) * 100;
            t.prob[(size_t)i * nB + b] = acc;
        }
        const float last = t.prob[(size_t)i * nB + nB - 1];
        for (int b = 0; b < nB; ++b) t.prob[(size_t)i * nB + b] = t.prob[(size_t)i * nB + b] / last;
    }
    t.probg.clear();
    t.wq.assign(1, 1.0f);
    t.ref_sampling = true;
    t.valid = true;
}

void fill_ib(HostTable &t) {
    if (!t.Ib.empty()) return;
    t.Ib.assign((size_t)t.nbands * t.nT, 0.f);
    for (int b = 0; b < t.nbands; ++b)
        for (int i = 0; i < t.nT; ++i) t.Ib[(size_t)b * t.nT + i] = planck_band(t.T0 + i * t.dT, t.wvc[b]);
}

// Clamped linear position (same as the kernel's grid_pos, in double).
void gpos(double v, double v0, double d, int n, int *i, double *f) {
    double p = (v - v0) / d;
    p = std::min(std::max(p, 0.0), (double)(n - 1));
    int ii = std::min((int)p, n - 2);
    if (n < 2) ii = 0;
    *i = ii;
    *f = p - ii;
}

double k_at(const HostTable &t, int b, int g, double T, double x) {
    int ti, xi = 0;
    double ft, fx = 0.0;
    gpos(T, t.T0, t.dT, t.nT, &ti, &ft);
    const float *s = t.k.data() + ((size_t)b * t.nq + g) * t.nT * t.nX;
    if (t.nX > 1) {
        gpos(x, t.X0, t.dX, t.nX, &xi, &fx);
        const double k0 = s[ti * t.nX + xi] + fx * (s[ti * t.nX + xi + 1] - s[ti * t.nX + xi]);
        const double k1 = s[(ti + 1) * t.nX + xi] + fx * (s[(ti + 1) * t.nX + xi + 1] - s[(ti + 1) * t.nX + xi]);
        return k0 + ft * (k1 - k0);
    }
    return s[ti] + ft * (s[ti + 1] - s[ti]);
}

double ib_at(const HostTable &t, int b, double T) {
    int ti;
    double ft;
    gpos(T, t.T0, t.dT, t.nT, &ti, &ft);
    const float *s = t.Ib.data() + (size_t)b * t.nT;
    return s[ti] + ft * (s[ti + 1] - s[ti]);
}

// Vose alias table over K probabilities, thresholds quantised to 2^-24, then
// the exact sampling probability of every entry as the kernel draws it:
// slot j = floor(x*K / 2^32) for a 32-bit x, accept slot j when
// (y>>8)*2^-24 < thr_j, else take alias_j.
void build_alias(const std::vector<double> &q, std::vector<float> &thr, std::vector<int> &alias,
                 std::vector<double> &peff) {
    const int K = (int)q.size();
    thr.assign(K, 1.0f);
    alias.resize(K);
    for (int j = 0; j < K; ++j) alias[j] = j;
    std::vector<double> sc(K);
    double tot = 0.0;
    for (double v : q) tot += v;
    std::vector<int> small, large;
    for (int j = 0; j < K; ++j) {
        sc[j] = q[j] / tot * K;
        (sc[j] < 1.0 ? small : large).push_back(j);
    }
    std::vector<double> pr(K, 1.0);
    while (!small.empty() && !large.empty()) {
        const int s = small.back(); small.pop_back();
        const int l = large.back(); large.pop_back();
        pr[s] = sc[s];
        alias[s] = l;
        sc[l] = (sc[l] + sc[s]) - 1.0;
        (sc[l] < 1.0 ? small : large).push_back(l);
    }
    for (int j : large) pr[j] = 1.0;
    for (int j : small) pr[j] = 1.0;
    peff.assign(K, 0.0);
    const double two32 = 4294967296.0, two24 = 16777216.0;
    for (int j = 0; j < K; ++j) {
        double m = ceil(pr[j] * two24);
        if (m > two24) m = two24;
        if (m < 0) m = 0;
        thr[j] = (float)(m / two24);
        const double pacc = m / two24;
        // number of 32-bit x with floor(x*K/2^32) == j
        const double lo = ceil(j * two32 / K), hi = ceil((j + 1) * two32 / K);
        const double pslot = (hi - lo) / two32;
        peff[j] += pslot * pacc;
        peff[alias[j]] += pslot * (1.0 - pacc);
    }
}

int build_sampling(dnsmc_solver *s, float Tmax, float xm) {
    HostTable &t = s->tab;
    const dnsmc_config &c = s->cfg;
    s->entries.clear();
    s->group_start.clear();
    s->group_empty.clear();
    if (c.model == DNSMC_MODEL_GREY) {
        s->n_groups_used = 1;
        s->n_tbins_used = 1;
        s->group_start = {0, 0};
        s->group_empty = {0};
        return DNSMC_OK;
    }
    fill_ib(t);
    const int nB = t.nbands, nQ = t.nq;
    const int nG = std::min(c.n_groups, nB);
    s->n_groups_used = nG;
    const double Tm = Tmax;
    // Target coefficient C_s of every spectral sample s = (band, g): the group
    // estimate is sum_s C_s k(T_i) Ib(T_i) E[D | s], drawn with density q and
    // weighted W_s = C_s / q_eff(s).
    std::vector<double> C((size_t)nB * nQ, 0.0);
    if (t.ref_sampling) {
        // nearest table temperature to Tmax (code/mc_gpu.cu:142, :837)
        int tm = (int)((Tmax - t.T0) / t.dT);
        tm = std::max(0, std::min(tm, t.nT - 2));
        const float Tt0 = t.T0 + tm * t.dT, Tt1 = t.T0 + (tm + 1) * t.dT;
        const int ts = ((Tmax - Tt0) < (Tt1 - Tmax)) ? tm : tm + 1;
        // kappamax: Planck mean at Tmax (code/read_tables.cpp:334-336)
        int tk = (int)((Tmax - t.T0) / t.dT);
        tk = std::max(0, std::min(tk, t.nT - 2));
        const double kmax = (double)(t.kP[tk + 1] - t.kP[tk]) / t.dT * (Tmax - (t.T0 + tk * t.dT)) + t.kP[tk];
        const double E = 4.0 * kmax * kSigma * Tm * Tm * Tm * Tm;
        std::vector<double> pr((size_t)nB * nQ, 0.0);
        double tot = 0.0;
        for (int b = 0; b < nB; ++b) {
            const double pb = (double)t.prob[(size_t)ts * nB + b] - (b ? (double)t.prob[(size_t)ts * nB + b - 1] : 0.0);
            for (int g = 0; g < nQ; ++g) {
                double pg = (g == 0) ? 1.0 : 0.0;
                if (!t.probg.empty()) {
                    const float *cg = t.probg.data() + ((size_t)ts * nB + b) * nQ;
                    pg = (double)cg[g] - (g ? (double)cg[g - 1] : 0.0);
                }
                pr[(size_t)b * nQ + g] = std::max(0.0, pb) * std::max(0.0, pg);
                tot += pr[(size_t)b * nQ + g];
            }
        }
        if (!(tot > 0)) return fail(DNSMC_ERR_TABLE, "band CDF at T=%g is empty", (double)(t.T0 + ts * t.dT));
        for (int b = 0; b < nB; ++b)
            for (int g = 0; g < nQ; ++g) {
                const size_t s_ = (size_t)b * nQ + g;
                if (pr[s_] <= 0) continue;
                const double den = ib_at(t, b, Tm) * k_at(t, b, g, Tm, xm);
                // ray weight of the reference: Ibmax*ratioI = E * k_i Ib_i / (k_m Ib_m)
                C[s_] = den > 0 ? pr[s_] / tot * E / den : 0.0;
            }
    } else {
        for (int b = 0; b < nB; ++b)
            for (int g = 0; g < nQ; ++g) C[(size_t)b * nQ + g] = 4.0 * kPi * 100.0 * t.dnu[b] * t.wq[g];
    }
    s->Ccoef = C;
    s->cv_grp.assign(1, 0);
    s->cv_sid.clear();
    s->cv_C.clear();
    for (int G = 0; G < nG; ++G) {
        const int b0 = (int)((long long)G * nB / nG), b1 = (int)((long long)(G + 1) * nB / nG);
        for (int b = b0; b < b1; ++b)
            for (int g = 0; g < nQ; ++g)
                if (C[(size_t)b * nQ + g] > 0) { s->cv_sid.push_back(b * nQ + g); s->cv_C.push_back(C[(size_t)b * nQ + g]); }
        s->cv_grp.push_back((int)s->cv_sid.size());
    }
    // sampling temperatures: Tmax only, or every table temperature
    std::vector<double> Tbins;
    if (c.local_sampling) for (int i = 0; i < t.nT; ++i) Tbins.push_back(t.T0 + (double)i * t.dT);
    else Tbins.push_back(Tm);
    s->n_tbins_used = (int)Tbins.size();
    s->group_start.push_back(0);
    std::vector<double> q((size_t)nB * nQ);
    for (size_t ib = 0; ib < Tbins.size(); ++ib) {
        double mean = 0.0;
        int npos = 0;
        for (int b = 0; b < nB; ++b)
            for (int g = 0; g < nQ; ++g) {
                const size_t s_ = (size_t)b * nQ + g;
                const double kp = s->part.empty() ? 0.0 : s->fv_mean * (double)s->part[(size_t)b].x;
                q[s_] = C[s_] > 0 ? C[s_] * (k_at(t, b, g, Tbins[ib], xm) + kp) * ib_at(t, b, Tbins[ib]) : 0.0;
                if (C[s_] > 0) { mean += q[s_]; ++npos; }
            }
        mean /= std::max(1, npos);
        // floor keeps every sample with a non-zero coefficient reachable
        for (size_t s_ = 0; s_ < q.size(); ++s_)
            if (C[s_] > 0) q[s_] = std::max(q[s_], 1e-6 * mean);
        for (int G = 0; G < nG; ++G) {
            const int b0 = (int)((long long)G * nB / nG), b1 = (int)((long long)(G + 1) * nB / nG);
            std::vector<double> qg;
            std::vector<int> ids;
            for (int b = b0; b < b1; ++b)
                for (int g = 0; g < nQ; ++g)
                    if (q[(size_t)b * nQ + g] > 0) { qg.push_back(q[(size_t)b * nQ + g]); ids.push_back(b * nQ + g); }
            if (ib == 0) s->group_empty.push_back(qg.empty() ? 1 : 0);
            if (qg.size() > 65535) return fail(DNSMC_ERR_TABLE, "band group has more than 65535 samples");
            if (!qg.empty()) {
                std::vector<float> thr;
                std::vector<int> al;
                std::vector<double> peff;
                build_alias(qg, thr, al, peff);
                for (size_t j = 0; j < qg.size(); ++j) {
                    const int sid = ids[j];
                    const int b = sid / nQ, g = sid % nQ;
                    SpecEntry e;
                    e.prob = thr[j];
                    e.alias_nb = (uint32_t)al[j] | ((uint32_t)b << 16);
                    e.koff = (int32_t)sid;
                    e.W = peff[j] > 0 ? (float)(C[sid] / peff[j]) : 0.0f;
                    s->entries.push_back(e);
                }
            }
            s->group_start.push_back((int)s->entries.size());
        }
    }
    s->ibw.assign((size_t)2 * nB, 0.f);
    for (int b = 0; b < nB; ++b) {
        s->ibw[b] = planck_band(c.T_west, t.wvc[b]);
        s->ibw[nB + b] = planck_band(c.T_east, t.wvc[b]);
    }
    return DNSMC_OK;
}

int upload_tables(dnsmc_solver *s) {
    HostTable &t = s->tab;
    fill_ib(t);
    TRY(s->d_k.ensure(t.k.size()));
    TRY(s->d_ib.ensure(t.Ib.size()));
    CUDA_TRY(cudaMemcpyAsync(s->d_k.p, t.k.data(), t.k.size() * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(cudaMemcpyAsync(s->d_ib.p, t.Ib.data(), t.Ib.size() * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    // the march's per-sample slabs of paired values (value, difference to the
    // next): k over [t][x] -- rows t and t+1 side by side, one 16-byte entry
    // per table cell -- (or over [t]), then Ib over [t] of the sample's band
    const int nS = t.nbands * t.nq;
    const int klen = t.nX > 1 ? 2 * (t.nT - 1) * (t.nX - 1) : t.nT - 1;
    const int len = (klen + (t.nT - 1) + 1) & ~1;
    std::vector<float2> sl((size_t)nS * len, make_float2(0.f, 0.f));
    for (int sid = 0; sid < nS; ++sid) {
        float2 *o = sl.data() + (size_t)sid * len;
        if (t.nX > 1) {
            for (int ti = 0; ti < t.nT - 1; ++ti)
                for (int xi = 0; xi < t.nX - 1; ++xi) {
                    const float *r = t.k.data() + ((size_t)sid * t.nT + ti) * t.nX + xi;
                    const float *r1 = r + t.nX;
                    const int e = ti * (t.nX - 1) + xi;
                    o[2 * e] = make_float2(r[0], r[1] - r[0]);
                    o[2 * e + 1] = make_float2(r1[0], r1[1] - r1[0]);
                }
        } else {
            for (int ti = 0; ti < t.nT - 1; ++ti) {
                const float *r = t.k.data() + (size_t)sid * t.nT + ti;
                o[ti] = make_float2(r[0], r[1] - r[0]);
            }
        }
        const float *ib = t.Ib.data() + (size_t)(sid / t.nq) * t.nT;
        for (int ti = 0; ti < t.nT - 1; ++ti) o[klen + ti] = make_float2(ib[ti], ib[ti + 1] - ib[ti]);
    }
    TRY(s->d_slab.ensure(sl.size()));
    CUDA_TRY(cudaMemcpyAsync(s->d_slab.p, sl.data(), sl.size() * sizeof(float2), cudaMemcpyHostToDevice, s->stream));
    s->slab_len = len;
    s->slab_klen = klen;
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->tables_dirty = false;
    return DNSMC_OK;
}

int region_dims(const dnsmc_solver *s, int *ni, int *nj, int *nk) {
    *ni = s->r_i1 - s->r_i0;
    *nj = s->r_j1 - s->r_j0;
    *nk = s->r_k1 - s->r_k0;
    return DNSMC_OK;
}

// Cells per lane of the march: kLaneCells on the fine grid (absorbing gas
// with black walls, and the general medium with particles / grey walls), 1
// for the multigrid march (32-cell packets).
int lane_cells(const dnsmc_solver *s) {
    return s->cfg.grid_num > 1 ? 1 : kLaneCells;
}

// Packet tiling of the region: tile_a cells along j (a divisor of 32), by
// tile_b = 32 * lane_cells / tile_a along k.  Automatic: square 8 x 8
// packets for the two-cell march (its cells lie closest together: more even
// costs inside a packet for the per-packet ray counts, fewer idle lanes),
// 16 x 4 or 32 x 2 when k has fewer than 8 / 4 cells; the widest row that
// fits for the one-cell multigrid march.
void tiling(const dnsmc_solver *s, int *ta, int *tb, int *npa, int *npb, int *npw) {
    int ni, nj, nk;
    region_dims(s, &ni, &nj, &nk);
    int a = s->cfg.tile_a;
    if (!a) a = lane_cells(s) > 1 ? (nk >= 8 ? 8 : (nk >= 4 ? 16 : 32)) : (nj >= 32 ? 32 : (nj >= 16 ? 16 : 8));
    *ta = a;
    *tb = 32 / a * lane_cells(s);
    *npa = (nj + a - 1) / a;
    *npb = (nk + *tb - 1) / *tb;
    *npw = ni;
}

int solve_enqueue(dnsmc_solver *s, bool trace, int tf, int tg, int tp, int tr, int tmax_steps,
                  int *d_trace_rec, int *d_trace_n, unsigned int *d_trace_rng) {
    dnsmc_config &c = s->cfg;
    if (s->nfields < 1) return fail(DNSMC_ERR_STATE, "no fields: call dnsmc_set_fields first");
    if (c.model != DNSMC_MODEL_GREY && !s->tab.valid && !s->tab.grey_bands)
        return fail(DNSMC_ERR_STATE, "no tables: load or set tables first");
    TRY(set_device(s));
    const float Tmax = std::max(s->tmax_fields, std::max(c.T_west, c.T_east));
    const float xm = s->have_x ? (float)(s->xsum / ((double)s->nfields * c.imax * c.jmax * c.kmax)) : 0.f;
    if (!trace) {
        CUDA_TRY(cudaEventRecord(s->ev_solve0, s->stream));
        s->tmax_used = Tmax;
        // the sampling tables depend on these, the tables and the particle
        // optics only; rebuilding them is host work the device would wait for
        const double skey[8] = {(double)Tmax, (double)xm, s->fv_mean, (double)c.n_groups, (double)c.local_sampling,
                                (double)c.T_west, (double)c.T_east, (double)c.model};
        const bool reuse = s->sampling_valid && !s->tables_dirty && !s->tab.grey_bands &&
                           memcmp(skey, s->sampling_key, sizeof skey) == 0 && s->part.size() == s->sampling_part.size() &&
                           (s->part.empty() ||
                            memcmp(s->part.data(), s->sampling_part.data(), s->part.size() * sizeof(float2)) == 0);
        if (!reuse) {
            s->sampling_valid = false;
            if (s->tab.grey_bands) { build_grey_band_tables(s->tab, Tmax); s->tables_dirty = true; }
            TRY(build_sampling(s, Tmax, xm));
            if (c.model != DNSMC_MODEL_GREY && s->tables_dirty) TRY(upload_tables(s));
            if (c.model != DNSMC_MODEL_GREY) {
                TRY(s->d_entries.ensure(std::max<size_t>(1, s->entries.size())));
                TRY(s->d_ibw.ensure(s->ibw.size()));
                CUDA_TRY(cudaMemcpyAsync(s->d_entries.p, s->entries.data(), s->entries.size() * sizeof(SpecEntry), cudaMemcpyHostToDevice, s->stream));
                CUDA_TRY(cudaMemcpyAsync(s->d_ibw.p, s->ibw.data(), s->ibw.size() * sizeof(float), cudaMemcpyHostToDevice, s->stream));
            }
            TRY(s->d_group_start.ensure(s->group_start.size()));
            TRY(s->d_group_empty.ensure(s->group_empty.size()));
            CUDA_TRY(cudaMemcpyAsync(s->d_group_start.p, s->group_start.data(), s->group_start.size() * sizeof(int), cudaMemcpyHostToDevice, s->stream));
            CUDA_TRY(cudaMemcpyAsync(s->d_group_empty.p, s->group_empty.data(), s->group_empty.size() * sizeof(int), cudaMemcpyHostToDevice, s->stream));
            memcpy(s->sampling_key, skey, sizeof skey);
            s->sampling_part = s->part;
            s->sampling_valid = true;
            s->cv_uploaded = false;
        }
    }
    const HostTable &t = s->tab;
    int ni, nj, nk, ta, tb, npa, npb, npw;
    region_dims(s, &ni, &nj, &nk);
    tiling(s, &ta, &tb, &npa, &npb, &npw);
    MarchParams P;
    memset(&P, 0, sizeof P);  // the bytes form the graph key: padding included
    P.nw = c.imax; P.na = c.jmax; P.nb = c.kmax;
    P.da = s->da; P.db = s->db; P.fw = s->d_fw.p;
    P.ew0 = s->r_i0; P.ew1 = s->r_i1; P.ea0 = s->r_j0; P.ea1 = s->r_j1; P.eb0 = s->r_k0; P.eb1 = s->r_k1;
    P.tile_a = ta; P.tile_b = tb; P.npa = npa; P.npb = npb; P.npw = npw;
    P.n_packets = npa * npb * npw;
    P.nfields = s->nfields;
    P.field_stride = (long long)c.imax * c.jmax * c.kmax;
    int mode = MODE_GREY;
    if (c.model != DNSMC_MODEL_GREY) mode = (t.nX > 1) ? MODE_TX : MODE_T;
    s->mode = mode;
    P.fieldT = (mode == MODE_GREY) ? s->d_fieldT.p : nullptr;
    if (mode == MODE_TX && !s->have_x) return fail(DNSMC_ERR_STATE, "table has an x_H2O axis but fields were set without x");
    if (mode != MODE_TX && s->have_x)
        return fail(DNSMC_ERR_STATE, "fields carry x_H2O but the spectral model has no x axis: set fields without x");
    P.nbands = t.nbands; P.nT = t.nT; P.nX = t.nX;
    P.T0 = t.T0; P.invdT = 1.0f / t.dT; P.X0 = t.X0; P.invdX = 1.0f / t.dX;
    if (mode != MODE_GREY) { P.slab = s->d_slab.p; P.slab_len = s->slab_len; P.slab_klen = s->slab_klen; }
    // polls of the first bounded wait for a ray's slab copy; the environment
    // variable DNSMC_TEST_SLAB_FIRST_POLLS lowers it only to drive the
    // time-out path in tests (0: every first wait runs out at once, the
    // second one receives the copy, and the solve reports DNSMC_ERR_TIMEOUT)
    P.slab_polls0 = kSlabWaitPolls;
    if (const char *ev = getenv("DNSMC_TEST_SLAB_FIRST_POLLS"))
        if (*ev) P.slab_polls0 = std::min(std::max(atoi(ev), 0), kSlabWaitPolls);
    P.ibw = s->d_ibw.p;
    P.entries = s->d_entries.p; P.group_start = s->d_group_start.p;
    P.n_groups = s->n_groups_used;
    P.n_tbins = s->n_tbins_used;
    P.sampler = c.sampler;
    P.nbatch = c.nvar;
    P.kappa = c.kappa;
    P.Wgrey = (float)(4.0 * c.kappa * kSigma);
    P.Tw4[0] = c.T_west * c.T_west * c.T_west * c.T_west;
    P.Tw4[1] = c.T_east * c.T_east * c.T_east * c.T_east;
    // general medium: particles (with their field) and/or grey walls
    const bool have_part = !s->part.empty();
    if (have_part && s->fv_fields != s->nfields)
        return fail(DNSMC_ERR_STATE, "particles set: set the particle field of the %d resident snapshots", s->nfields);
    const bool gen = have_part || c.eps_west < 1.0f || c.eps_east < 1.0f;
    P.fieldV = have_part ? s->d_fieldV.p : nullptr;
    P.part = have_part ? s->d_part.p : nullptr;
    P.fv_max = have_part ? s->fv_max : 0.0f;
    P.hg_g = s->hg_g;
    P.eps[0] = c.eps_west; P.eps[1] = c.eps_east;
    P.W4sig = (float)(4.0 * kSigma);
    // multigrid: the reference's plain estimator only
    const bool mg = c.grid_num > 1;
    if (mg) {
        if (mode == MODE_TX) return fail(DNSMC_ERR_STATE, "multigrid needs a table without an x_H2O axis");
        if (c.control_variate) return fail(DNSMC_ERR_STATE, "multigrid is not combined with the control variate");
        if (gen) return fail(DNSMC_ERR_STATE, "multigrid is not combined with particles or grey walls");
        if (s->mg_fields != s->nfields) return fail(DNSMC_ERR_STATE, "coarse fields missing: set the fields again");
        P.mg_levels = c.grid_num;
        P.mg_steps = c.mg_steps;
        P.mgT = s->d_mgT.p;
        P.mgfw = s->d_mgfw.p;
        for (int l = 1; l < c.grid_num; ++l) {
            P.mg_off[l] = s->mg_off[l];
            P.mg_fwoff[l] = s->mg_fwoff[l];
            P.mg_da[l] = c.Ly / (float)(c.jmax >> l);
            P.mg_db[l] = c.Lz / (float)(c.kmax >> l);
        }
        P.Ly = c.Ly;
        P.Lz = c.Lz;
    }
    P.rays = s->rays;
    const bool per_item = !s->rays_pp.empty() || s->rays_dev;
    P.rays_per_packet = per_item ? s->d_rays_pp.p : nullptr;
    P.rays_gstride = 0;
    P.key0 = (uint32_t)(c.seed & 0xffffffffu);
    P.key1 = (uint32_t)(c.seed >> 32);
    P.field_base = 0;
    P.toll = c.toll;
    P.dtoll = (float)(-log((double)c.toll));
    P.max_steps = c.max_steps;
    P.region_cells = (long long)ni * nj * nk;
    P.n_items = (long long)s->nfields * P.n_groups * P.n_packets;
    if (per_item && s->rays_np != P.n_packets)
        return fail(DNSMC_ERR_STATE,
                    "per-packet rays were set for %d packets, the solve has %d (the packet shape follows the "
                    "march: grid levels use 32-cell packets): set the rays again",
                    s->rays_np, P.n_packets);
    if (per_item && s->rays_pg > 0) {
        if (s->rays_pg != P.n_groups)
            return fail(DNSMC_ERR_STATE, "per-item ray table has %d band groups, the solve has %d", s->rays_pg,
                         P.n_groups);
        P.rays_gstride = P.n_packets;
    }
    const long long ncell = (long long)s->nfields * P.field_stride;
    if (mode == MODE_TX && !trace) TRY(s->d_posTX.ensure((size_t)ncell));
    if (mode == MODE_T && !trace) TRY(s->d_posT.ensure((size_t)ncell));
    P.fieldP = s->d_posT.p;
    P.fieldPX = s->d_posTX.p;
    TRY(s->d_misc.ensure(4));
    TRY(s->d_counters.ensure(2));
    P.queue = s->d_misc.p;
    P.status = s->d_misc.p + 1;
    P.counters = s->d_counters.p;
    int threads = c.block_threads ? c.block_threads : 256;
    {
        // every warp holds its ray's table slab in shared memory
        int smax = 0;
        if (cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->device) != cudaSuccess)
            smax = 48 * 1024;
        const size_t stat = 1024;  // the march kernels' static shared memory (barriers), at most
        if (march_smem(P, threads, kLaneCells) + stat > (size_t)smax) threads = 128;
        if (march_smem(P, threads, kLaneCells) + stat > (size_t)smax)
            return fail(DNSMC_ERR_TABLE, "a spectral sample's table slab (%d bytes) exceeds the shared memory of the march",
                        P.slab_len * 8);
    }
    const bool cv = c.control_variate != 0;
    const int S = (mode == MODE_GREY) ? 1 : t.nbands * t.nq;
    if (cv) {
        P.n_samples = S;
        P.sur = s->d_sur.p;
        P.surtab = s->d_surtab.p;
        P.beta = s->beta_set ? s->d_beta.p : nullptr;
    }
    const bool mom = cv && c.cv_moments;
    if (trace) {
        // a trace reuses the surrogate of the last solve: it must cover the fields
        const size_t nsur = (size_t)s->nfields * S * c.imax;
        if (cv && (s->d_sur.n < nsur || s->d_surtab.n < nsur * 2 * kSurBins))
            return fail(DNSMC_ERR_STATE, "trace with the control variate needs a prior solve of these fields");
        P.trace_f = tf; P.trace_g = tg; P.trace_p = tp; P.trace_r = tr; P.trace_max = tmax_steps;
        P.trace_rec = d_trace_rec; P.trace_n = d_trace_n; P.trace_rng = d_trace_rng;
        P.tally = nullptr;
        const int rc = mg ? launch_march_mg(mode, P, 1, 32, s->stream, true)
                          : launch_march_ex(mode, P, 1, 32, s->stream, true, cv, false, gen);
        if (rc) return fail(DNSMC_ERR_CUDA, "trace launch: %s", cudaGetErrorString((cudaError_t)rc));
        return DNSMC_OK;
    }
    // ---- buffers and kernel parameters (no kernel is enqueued yet) ----------
    CvParams cp;
    memset(&cp, 0, sizeof cp);
    if (cv) {
        // E[Y] per (field, group, cell): layer means -> layer-mean medium ->
        // surrogate table and its means Jhat -> sum over the group's samples
        const size_t nsur = (size_t)s->nfields * S * c.imax;
        TRY(s->d_layer.ensure((size_t)s->nfields * c.imax));
        TRY(s->d_sur.ensure(nsur));
        TRY(s->d_surtab.ensure(nsur * 2 * kSurBins));
        TRY(s->d_Jhat.ensure(nsur));
        TRY(s->d_Jf.ensure(nsur));
        TRY(s->d_muY.ensure((size_t)s->nfields * P.n_groups * P.region_cells));
        if (mode != MODE_GREY && !s->cv_uploaded) {
            TRY(s->d_cv_grp.ensure(s->cv_grp.size()));
            TRY(s->d_cv_sid.ensure(std::max<size_t>(1, s->cv_sid.size())));
            TRY(s->d_cv_C.ensure(std::max<size_t>(1, s->cv_C.size())));
            CUDA_TRY(cudaMemcpyAsync(s->d_cv_grp.p, s->cv_grp.data(), s->cv_grp.size() * sizeof(int), cudaMemcpyHostToDevice, s->stream));
            CUDA_TRY(cudaMemcpyAsync(s->d_cv_sid.p, s->cv_sid.data(), s->cv_sid.size() * sizeof(int), cudaMemcpyHostToDevice, s->stream));
            CUDA_TRY(cudaMemcpyAsync(s->d_cv_C.p, s->cv_C.data(), s->cv_C.size() * sizeof(double), cudaMemcpyHostToDevice, s->stream));
            s->cv_Cf.assign(s->cv_C.begin(), s->cv_C.end());
            TRY(s->d_cv_Cf.ensure(std::max<size_t>(1, s->cv_Cf.size())));
            CUDA_TRY(cudaMemcpyAsync(s->d_cv_Cf.p, s->cv_Cf.data(), s->cv_Cf.size() * sizeof(float), cudaMemcpyHostToDevice, s->stream));
            s->cv_uploaded = true;
        }
        cp.nfields = s->nfields; cp.nw = c.imax; cp.na = c.jmax; cp.nb = c.kmax;
        cp.fieldT = (mode == MODE_TX) ? nullptr : s->d_fieldT.p;
        cp.fieldTX = (mode == MODE_TX) ? s->d_fieldTX.p : nullptr;
        cp.mode = mode;
        cp.layer = s->d_layer.p;
        cp.nbands = t.nbands; cp.nq = std::max(1, t.nq); cp.nT = t.nT; cp.nX = t.nX;
        cp.T0 = P.T0; cp.invdT = P.invdT; cp.X0 = P.X0; cp.invdX = P.invdX;
        cp.ktab = s->d_k.p; cp.ibtab = s->d_ib.p; cp.ibw = P.ibw;
        cp.kappa = c.kappa; cp.Tw4[0] = P.Tw4[0]; cp.Tw4[1] = P.Tw4[1];
        cp.n_samples = S; cp.sur = s->d_sur.p; cp.fw = s->d_fw.p; cp.toll = c.toll; cp.dtoll = P.dtoll;
        cp.surtab = s->d_surtab.p;
        cp.Jhat = s->d_Jhat.p;
        cp.Jf = s->d_Jf.p;
        cp.samp_Cf = s->d_cv_Cf.p;
        cp.n_groups = P.n_groups;
        cp.grp_start = s->d_cv_grp.p; cp.samp_id = s->d_cv_sid.p; cp.samp_C = s->d_cv_C.p;
        cp.Wgrey = 4.0 * c.kappa * kSigma;
        cp.ew0 = P.ew0; cp.ew1 = P.ew1; cp.ea0 = P.ea0; cp.ea1 = P.ea1; cp.eb0 = P.eb0; cp.eb1 = P.eb1;
        cp.region_cells = P.region_cells;
        cp.muY = s->d_muY.p;
        if (have_part) {
            TRY(s->d_layerV.ensure((size_t)s->nfields * c.imax));
            cp.fieldV = s->d_fieldV.p;
            cp.part = s->d_part.p;
            cp.layerV = s->d_layerV.p;
        }
        // E[Y] from node sums for tables without particles
        if (mode != MODE_GREY && !have_part) {
            TRY(s->d_cvnodes.ensure((size_t)cv_node_count(cp)));
            cp.nodes = s->d_cvnodes.p;
        }
        s->cv_samples = S;
        P.sur = s->d_sur.p;
        P.surtab = s->d_surtab.p;
        if (mom) {
            TRY(s->d_moments.ensure((size_t)s->nfields * P.n_groups * P.region_cells * 9));
            P.moments = s->d_moments.p;
        }
    }
    TRY(s->d_tally.ensure((size_t)s->nfields * P.n_groups * P.region_cells));
    P.tally = s->d_tally.p;
    TRY(s->d_item_steps.ensure((size_t)P.n_items));
    P.item_steps = s->d_item_steps.p;
    if (P.rays_per_packet) {  // uneven items: longest first
        TRY(s->d_order.ensure((size_t)P.n_items));
        TRY(s->d_order_hist.ensure(kOrderBuckets));
        P.item_order = s->d_order.p;
    }
    const int sms = device_sm_count();
    const size_t smem = march_smem(P, threads, mg ? 1 : kLaneCells);
    const int occ = mg ? march_mg_occupancy(mode, threads, smem) : march_occupancy_ex(mode, threads, cv, mom, gen, smem);
    const int blocks = std::max(1, sms * occ);

    FinalizeParams F;
    memset(&F, 0, sizeof F);
    F.nfields = s->nfields; F.n_groups = P.n_groups; F.region_cells = P.region_cells;
    F.niR = ni; F.njR = nj; F.nkR = nk;
    F.tile_a = ta; F.tile_b = tb; F.npa = npa; F.npb = npb;
    F.rays = s->rays; F.rays_per_packet = P.rays_per_packet; F.rays_gstride = P.rays_gstride;
    F.batched = c.sampler == DNSMC_SAMPLER_RQMC;
    F.nbatch = c.nvar;
    if (F.rays_per_packet) {
        TRY(s->d_rays_rcp.ensure((size_t)finalize_rcp_count(F)));
        F.rcp = s->d_rays_rcp.p;
    }
    F.group_empty = s->d_group_empty.p;
    F.tally = s->d_tally.p;
    F.muY = cv ? s->d_muY.p : nullptr;
    F.beta = cv ? P.beta : nullptr;
    const size_t nout = (size_t)s->nfields * P.region_cells;
    TRY(s->d_Q.ensure(nout));
    TRY(s->d_var.ensure(nout));
    TRY(s->d_sig.ensure(nout));
    TRY(s->d_Qg.ensure(nout * P.n_groups));
    TRY(s->d_varg.ensure(nout * P.n_groups));
    F.Q = s->d_Q.p; F.var = s->d_var.p; F.sigma = s->d_sig.p; F.Qg = s->d_Qg.p; F.varg = s->d_varg.p;
    F.status = P.status;
    const bool f32 = s->result_type == DNSMC_RESULT_F32;
    if (f32) {
        TRY(s->d_Qf.ensure(nout));
        TRY(s->d_sigf.ensure(nout));
        TRY(s->h_Qf.ensure(nout));
        TRY(s->h_sigf.ensure(nout));
        F.Qf = s->d_Qf.p; F.sigf = s->d_sigf.p; F.sig_scale = s->sig_scale;
    } else {
        TRY(s->h_Q.ensure(nout));
        TRY(s->h_sig.ensure(nout));
    }

    // ---- the kernel sequence of a solve (stream-ordered; capturable) -------
    auto kernels = [&](bool events) -> int {
        if (mode != MODE_GREY) {
            // table coordinates of the field for this table (once per solve)
            const int rcp = mode == MODE_TX
                                ? launch_field_pos(nullptr, s->d_fieldTX.p, nullptr, s->d_posTX.p, ncell, P.T0,
                                                   P.invdT, P.nT, P.X0, P.invdX, P.nX, s->stream)
                                : launch_field_pos(s->d_fieldT.p, nullptr, s->d_posT.p, nullptr, ncell, P.T0, P.invdT,
                                                   P.nT, P.X0, P.invdX, P.nX, s->stream);
            if (rcp) return fail(DNSMC_ERR_CUDA, "coordinate launch: %s", cudaGetErrorString((cudaError_t)rcp));
        }
        if (cv) {
            int rc = launch_cv_prepare(cp, s->stream);
            if (rc == 0) rc = launch_cv_mean(cp, s->stream);
            if (rc) return fail(DNSMC_ERR_CUDA, "control-variate launch: %s", cudaGetErrorString((cudaError_t)rc));
        }
        CUDA_TRY(cudaMemsetAsync(s->d_misc.p, 0, 4 * sizeof(unsigned int), s->stream));
        CUDA_TRY(cudaMemsetAsync(s->d_counters.p, 0, 2 * sizeof(unsigned long long), s->stream));
        if (P.item_order) {
            const int rco = launch_item_order(P.rays_per_packet, P.rays_gstride, P.n_packets, P.n_groups, P.n_items,
                                              std::max(1, c.sampler == DNSMC_SAMPLER_RQMC ? c.nvar : 1),
                                              s->d_order_hist.p, s->d_order.p, s->stream);
            if (rco) return fail(DNSMC_ERR_CUDA, "queue order launch: %s", cudaGetErrorString((cudaError_t)rco));
        }
        if (events) CUDA_TRY(cudaEventRecord(s->ev_march0, s->stream));
        int rc = mg ? launch_march_mg(mode, P, blocks, threads, s->stream, false)
                    : launch_march_ex(mode, P, blocks, threads, s->stream, false, cv, mom, gen);
        if (rc) return fail(DNSMC_ERR_CUDA, "march launch: %s", cudaGetErrorString((cudaError_t)rc));
        if (events) CUDA_TRY(cudaEventRecord(s->ev_march1, s->stream));
        rc = launch_finalize(F, s->stream);
        if (rc) return fail(DNSMC_ERR_CUDA, "finalize launch: %s", cudaGetErrorString((cudaError_t)rc));
        if (f32) {
            CUDA_TRY(cudaMemcpyAsync(s->h_Qf.p, s->d_Qf.p, nout * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
            CUDA_TRY(cudaMemcpyAsync(s->h_sigf.p, s->d_sigf.p, nout * sizeof(float), cudaMemcpyDeviceToHost,
                                     s->stream));
        } else {
            CUDA_TRY(cudaMemcpyAsync(s->h_Q.p, s->d_Q.p, nout * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
            CUDA_TRY(cudaMemcpyAsync(s->h_sig.p, s->d_sig.p, nout * sizeof(double), cudaMemcpyDeviceToHost,
                                     s->stream));
        }
        return DNSMC_OK;
    };

    if (!s->graph_on) {
        TRY(kernels(true));
    } else {
        // Replay the captured sequence when every parameter it baked in is
        // unchanged; otherwise capture it again.  The march timing then
        // brackets the whole graph.
        std::vector<unsigned char> key(sizeof P + sizeof cp + sizeof F + 4 * sizeof(long long));
        unsigned char *k = key.data();
        memcpy(k, &P, sizeof P); k += sizeof P;
        memcpy(k, &cp, sizeof cp); k += sizeof cp;
        memcpy(k, &F, sizeof F); k += sizeof F;
        const long long extra[4] = {blocks, threads, (long long)(cv ? 1 : 0) | (mom ? 2 : 0) | ((long long)mode << 2),
                                    (long long)(uintptr_t)s->stream};
        memcpy(k, extra, sizeof extra);
        if (!s->graph_exec || key != s->graph_key) {
            if (s->graph_exec) { cudaGraphExecDestroy(s->graph_exec); s->graph_exec = nullptr; }
            cudaGraph_t g = nullptr;
            CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeRelaxed));
            const long long counted = launch_count();
            const int rc = kernels(false);
            note_launch(counted - launch_count());  // captured, not launched: each replay counts them
            const cudaError_t ec = cudaStreamEndCapture(s->stream, &g);
            if (rc) { if (g) cudaGraphDestroy(g); return rc; }
            if (ec != cudaSuccess) return fail(DNSMC_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ec));
            // kernel nodes of the graph: the launches each replay adds
            size_t nn = 0;
            s->graph_kernels = 0;
            if (cudaGraphGetNodes(g, nullptr, &nn) == cudaSuccess && nn) {
                std::vector<cudaGraphNode_t> nodes(nn);
                if (cudaGraphGetNodes(g, nodes.data(), &nn) == cudaSuccess)
                    for (size_t q = 0; q < nn; ++q) {
                        cudaGraphNodeType ty;
                        if (cudaGraphNodeGetType(nodes[q], &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel)
                            s->graph_kernels += 1;
                    }
            }
            const cudaError_t ei = cudaGraphInstantiate(&s->graph_exec, g, 0);
            cudaGraphDestroy(g);
            if (ei != cudaSuccess) { s->graph_exec = nullptr; return fail(DNSMC_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ei)); }
            s->graph_key = key;
            s->graph_captures += 1;
        }
        CUDA_TRY(cudaEventRecord(s->ev_march0, s->stream));
        CUDA_TRY(cudaGraphLaunch(s->graph_exec, s->stream));
        CUDA_TRY(cudaEventRecord(s->ev_march1, s->stream));
        s->graph_launches += 1;
        note_launch(s->graph_kernels);
    }
    s->last = P;
    s->lastF = F;
    CUDA_TRY(cudaEventRecord(s->ev_done, s->stream));
    s->in_flight = true;
    s->solved = true;
    s->solved_result_type = s->result_type;
    return DNSMC_OK;
}

int wait_done(dnsmc_solver *s, double timeout_s) {
    if (!s->in_flight) return DNSMC_OK;
    TRY(set_device(s));
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t e = cudaEventQuery(s->ev_done);
        if (e == cudaSuccess) break;
        if (e != cudaErrorNotReady) return fail(DNSMC_ERR_CUDA, "solve failed: %s", cudaGetErrorString(e));
        if (timeout_s > 0) {
            const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (el > timeout_s) return fail(DNSMC_ERR_TIMEOUT, "solve still running after %.3f s", timeout_s);
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    s->in_flight = false;
    CUDA_TRY(cudaEventElapsedTime(&s->march_ms, s->ev_march0, s->ev_march1));
    CUDA_TRY(cudaEventElapsedTime(&s->solve_ms, s->ev_solve0, s->ev_done));
    unsigned int misc[4];
    CUDA_TRY(cudaMemcpy(misc, s->d_misc.p, sizeof misc, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(s->h_counters, s->d_counters.p, sizeof s->h_counters, cudaMemcpyDeviceToHost));
    s->h_status = misc[1];
    if (s->h_status & DNSMC_STATUS_COPY_TIMEOUT)
        return fail(DNSMC_ERR_TIMEOUT, "solve failed: a march's table copy did not arrive within its bounded wait");
    return DNSMC_OK;
}

// Coarse temperatures of every field for the multigrid march: the spline
// coarsening (interp3D) on the device from the packed fine temperatures
// (src: [f][i][k][j], T every src_step floats), three passes per level and
// field on the solver's stream; the coarse wall-normal faces of every level.
int upload_coarse(dnsmc_solver *s, int nfields, const float *src, int src_step) {
    const dnsmc_config &c = s->cfg;
    const int G = c.grid_num;
    const int I = c.imax, J = c.jmax, K = c.kmax;
    const long long ncell = (long long)I * J * K;
    long long off = 0;
    for (int l = 1; l < G; ++l) {
        s->mg_off[l] = off;
        off += (long long)nfields * (I >> l) * (J >> l) * (K >> l);
    }
    // cell-centre positions, 1-based: fine x, y, z, then per level coarse x, y, z
    std::vector<float> xu, yu, zu, pos, cen;
    make_faces(I, c.Lx, c.stretched_x, xu);
    uniform_faces(J, c.Ly, yu);
    uniform_faces(K, c.Lz, zu);
    long long po[kMaxLevels][3] = {}, pf[3];
    auto put = [&](const std::vector<float> &u) {
        centres(u, cen);
        const long long o = (long long)pos.size();
        pos.insert(pos.end(), cen.begin(), cen.end());
        return o;
    };
    pf[0] = put(xu); pf[1] = put(yu); pf[2] = put(zu);
    std::vector<float> faces;
    int fo = 0;
    for (int l = 1; l < G; ++l) {
        std::vector<float> cxu, cyu, czu;
        coarse_faces(I, l, c.Lx, c.stretched_x, cxu);
        uniform_faces(J >> l, c.Ly, cyu);
        uniform_faces(K >> l, c.Lz, czu);
        po[l][0] = put(cxu); po[l][1] = put(cyu); po[l][2] = put(czu);
        s->mg_fwoff[l] = fo;
        faces.insert(faces.end(), cxu.begin(), cxu.end());
        fo += (int)cxu.size();
    }
    const int im1 = I >> 1, jm1 = J >> 1;
    const long long ntmp = (long long)im1 * J * K + (long long)im1 * jm1 * K;  // level 1 is the largest
    const long long nwork = 3 * std::max({(long long)(I + 2) * J * K, (long long)(J + 2) * im1 * K,
                                          (long long)(K + 2) * im1 * jm1});
    TRY(s->d_mgT.ensure((size_t)std::max(1LL, off)));
    TRY(s->d_mgfw.ensure(faces.size()));
    TRY(s->d_mgpos.ensure(pos.size()));
    TRY(s->d_mgtmp.ensure((size_t)(ntmp + nwork)));
    CUDA_TRY(cudaMemcpyAsync(s->d_mgfw.p, faces.data(), faces.size() * sizeof(float), cudaMemcpyHostToDevice,
                             s->stream));
    CUDA_TRY(cudaMemcpyAsync(s->d_mgpos.p, pos.data(), pos.size() * sizeof(float), cudaMemcpyHostToDevice,
                             s->stream));
    const float *P = s->d_mgpos.p;
    float *tx = s->d_mgtmp.p;
    float *work = tx + ntmp;
    for (int f = 0; f < nfields; ++f)
        for (int l = 1; l < G; ++l) {
            const int im = I >> l, jm = J >> l, km = K >> l;
            float *txy = tx + (long long)im * J * K;
            SplinePass q{};
            q.work = work;
            // along x: fine [i][k][j] -> tx [ic][k][j], lines (j, k)
            q.src = src + (long long)f * ncell * src_step; q.src_step = src_step;
            q.s_a = 1; q.s_b = J; q.s_e = (long long)J * K;
            q.dst = tx; q.d_a = 1; q.d_b = J; q.d_e = (long long)J * K;
            q.na = J; q.nlines = (long long)J * K; q.n = I; q.m = im;
            q.xf = P + pf[0]; q.xc = P + po[l][0];
            int rc = launch_spline_pass(q, s->stream);
            // along y: tx [ic][k][j] -> txy [ic][k][jc], lines (ic, k)
            if (!rc) {
                q.src = tx; q.src_step = 1;
                q.s_a = (long long)K * J; q.s_b = J; q.s_e = 1;
                q.dst = txy; q.d_a = (long long)K * jm; q.d_b = jm; q.d_e = 1;
                q.na = im; q.nlines = (long long)im * K; q.n = J; q.m = jm;
                q.xf = P + pf[1]; q.xc = P + po[l][1];
                rc = launch_spline_pass(q, s->stream);
            }
            // along z: txy [ic][k][jc] -> the march layout [ic][kc][jc], lines (jc, ic)
            if (!rc) {
                q.src = txy;
                q.s_a = 1; q.s_b = (long long)K * jm; q.s_e = jm;
                q.dst = s->d_mgT.p + s->mg_off[l] + (long long)f * im * jm * km;
                q.d_a = 1; q.d_b = (long long)km * jm; q.d_e = jm;
                q.na = jm; q.nlines = (long long)jm * im; q.n = K; q.m = km;
                q.xf = P + pf[2]; q.xc = P + po[l][2];
                rc = launch_spline_pass(q, s->stream);
            }
            if (rc) return fail(DNSMC_ERR_CUDA, "spline coarsening launch: %s", cudaGetErrorString((cudaError_t)rc));
        }
    s->mg_fields = nfields;
    return DNSMC_OK;
}

// Tmax / Tmin / sum x over the packed resident fields (code/mc_gpu.cu:470-486),
// on the device; fails (and drops the fields) when a temperature is not
// positive and finite.
int field_stats_checked(dnsmc_solver *s, int nfields, bool with_x, double st[4]) {
    const dnsmc_config &c = s->cfg;
    const long long ncell = (long long)c.imax * c.jmax * c.kmax;
    TRY(s->d_stat_part.ensure(field_stats_partials()));
    TRY(s->d_stat_out.ensure(4));
    const int rc = launch_field_stats(with_x ? nullptr : s->d_fieldT.p, with_x ? s->d_fieldTX.p : nullptr,
                                      nfields * ncell, s->d_stat_part.p, s->d_stat_out.p, s->stream);
    if (rc) return fail(DNSMC_ERR_CUDA, "stats launch: %s", cudaGetErrorString((cudaError_t)rc));
    CUDA_TRY(cudaMemcpyAsync(st, s->d_stat_out.p, 4 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (st[3] > 0.0 || !(st[1] > 0.0) || !std::isfinite(st[0])) {
        s->nfields = 0;
        return fail(DNSMC_ERR_ARG, "temperature field has non-positive or non-finite values");
    }
    return DNSMC_OK;
}

int upload_fields_host(dnsmc_solver *s, int nfields, const float *T, const float *x, int layout) {
    const dnsmc_config &c = s->cfg;
    const long long ncell = (long long)c.imax * c.jmax * c.kmax;
    long long si = 1, sj, sk, base, nsrc;
    if (layout == DNSMC_LAYOUT_DENSE) {
        sj = c.imax; sk = (long long)c.imax * c.jmax; base = 0; nsrc = ncell;
    } else if (layout == DNSMC_LAYOUT_FORTRAN) {
        sj = c.imax + 2; sk = (long long)(c.imax + 2) * (c.jmax + 2);
        base = 1 + sj + sk;
        nsrc = (long long)(c.imax + 2) * (c.jmax + 2) * (c.kmax + 2);
    } else {
        return fail(DNSMC_ERR_ARG, "unknown layout %d", layout);
    }
    TRY(set_device(s));
    TRY(wait_done(s, 0));
    const bool want_x = (x != nullptr);
    TRY(s->d_raw.ensure((size_t)nsrc * (want_x ? 2 : 1)));
    if (want_x) TRY(s->d_fieldTX.ensure((size_t)nfields * ncell));
    else TRY(s->d_fieldT.ensure((size_t)nfields * ncell));
    // each snapshot straight from the caller's arrays into the raw buffer
    // (stream order serialises the buffer's reuse), then packed on the device
    for (int f = 0; f < nfields; ++f) {
        CUDA_TRY(cudaMemcpyAsync(s->d_raw.p, T + f * nsrc, nsrc * sizeof(float), cudaMemcpyHostToDevice, s->stream));
        if (want_x)
            CUDA_TRY(cudaMemcpyAsync(s->d_raw.p + nsrc, x + f * nsrc, nsrc * sizeof(float), cudaMemcpyHostToDevice,
                                     s->stream));
        int rc;
        if (want_x)
            rc = launch_pack_TX(s->d_raw.p, s->d_raw.p + nsrc, s->d_fieldTX.p + f * ncell, c.imax, c.jmax, c.kmax, si, sj, sk, base, s->stream);
        else
            rc = launch_pack_T(s->d_raw.p, s->d_fieldT.p + f * ncell, c.imax, c.jmax, c.kmax, si, sj, sk, base, s->stream);
        if (rc) return fail(DNSMC_ERR_CUDA, "pack launch: %s", cudaGetErrorString((cudaError_t)rc));
    }
    double st[4];
    TRY(field_stats_checked(s, nfields, want_x, st));
    if (c.grid_num > 1)
        TRY(upload_coarse(s, nfields, want_x ? (const float *)s->d_fieldTX.p : s->d_fieldT.p, want_x ? 2 : 1));
    s->nfields = nfields;
    s->have_x = want_x;
    s->tmax_fields = (float)st[0];
    s->tmin_fields = (float)st[1];
    s->xsum = st[2];
    return DNSMC_OK;
}

std::mutex g_dropin_mu;
dnsmc_solver *g_dropin = nullptr;
std::string g_dropin_tables;
dnsmc_config g_dropin_cfg;
bool g_dropin_cfg_set = false;

[[noreturn]] void dropin_die(const char *where) {
    fprintf(stderr, "Fatal error: %s (%s)\n*** FAILED - ABORTING\n", where, dnsmc_last_error());
    exit(1);
}

}  // namespace

namespace dnsmc {
// Error reporting for the other translation units of the library.
int report_error(int code, const char *msg) { return fail(code, "%s", msg); }

int solver_view(dnsmc_solver *s, SolverView *v) {
    if (!s || !v) return fail(DNSMC_ERR_ARG, "null argument");
    if (s->nfields < 1) return fail(DNSMC_ERR_STATE, "no fields: call dnsmc_set_fields first");
    TRY(set_device(s));
    const dnsmc_config &c = s->cfg;
    SolverView w{};
    w.device = s->device;
    w.stream = s->stream;
    w.model = c.model;
    w.mode = c.model == DNSMC_MODEL_GREY ? MODE_GREY : (s->tab.nX > 1 ? MODE_TX : MODE_T);
    w.imax = c.imax; w.jmax = c.jmax; w.kmax = c.kmax; w.nfields = s->nfields;
    w.n_groups = c.model == DNSMC_MODEL_GREY ? 1 : std::min(c.n_groups, std::max(1, s->tab.nbands));
    w.nvar = c.nvar; w.sampler = c.sampler;
    w.i0 = s->r_i0; w.i1 = s->r_i1; w.j0 = s->r_j0; w.j1 = s->r_j1; w.k0 = s->r_k0; w.k1 = s->r_k1;
    tiling(s, &w.tile_a, &w.tile_b, &w.npa, &w.npb, &w.npw);
    w.n_packets = w.npa * w.npb * w.npw;
    w.region_cells = (long long)(w.i1 - w.i0) * (w.j1 - w.j0) * (w.k1 - w.k0);
    w.field_stride = (long long)c.imax * c.jmax * c.kmax;
    w.fieldT = s->d_fieldT.p;
    w.fieldTX = s->d_fieldTX.p;
    w.fw = s->d_fw.p;
    if (c.model != DNSMC_MODEL_GREY) {
        w.T_lo = s->tab.T0; w.T_hi = s->tab.T0 + (s->tab.nT - 1) * s->tab.dT;
        w.X_lo = s->tab.X0; w.X_hi = s->tab.X0 + (s->tab.nX - 1) * s->tab.dX;
    }
    w.solved = s->solved ? 1 : 0;
    if (s->solved) {
        w.last_groups = s->last.n_groups;
        w.moments = (c.control_variate && c.cv_moments) ? s->d_moments.p : nullptr;
        w.varg = s->d_varg.p;
        w.item_steps = s->d_item_steps.p;
        w.rays = s->last.rays;
        w.rays_item = s->last.rays_per_packet;
        w.rays_gstride = s->last.rays_gstride;
    }
    *v = w;
    return DNSMC_OK;
}

int solver_beta_device(dnsmc_solver *s, float2 **beta, long long *n) {
    SolverView v;
    TRY(solver_view(s, &v));
    TRY(wait_done(s, 0));
    const long long m = (long long)v.nfields * v.n_groups * v.region_cells;
    TRY(s->d_beta.ensure((size_t)m));
    s->beta_set = true;
    *beta = s->d_beta.p;
    *n = m;
    return DNSMC_OK;
}

int solver_rays_device(dnsmc_solver *s, int n_groups, int **rays) {
    if (n_groups < 1) return fail(DNSMC_ERR_ARG, "n_groups must be >= 1");
    TRY(set_device(s));
    TRY(wait_done(s, 0));
    int np;
    TRY(dnsmc_packet_count(s, &np));
    TRY(s->d_rays_pp.ensure((size_t)n_groups * np));
    s->rays_pp.clear();
    s->rays_pg = n_groups;
    s->rays_dev = true;
    s->rays_np = np;
    *rays = s->d_rays_pp.p;
    return DNSMC_OK;
}
}  // namespace dnsmc

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char *dnsmc_last_error(void) { return g_err.c_str(); }
const char *dnsmc_version(void) { return "dnsmc-gb300 0.1 (sm_103a)"; }

void dnsmc_set_default_config(dnsmc_config *c) {
    if (!c) return;
    memset(c, 0, sizeof *c);
    c->imax = 64; c->jmax = 64; c->kmax = 64; c->p_row = 1;
    c->Lx = 1.f; c->Ly = 1.f; c->Lz = 1.f;
    c->stretched_x = 1;
    c->nvar = 3; c->photmax = 20000;
    c->T_west = 500.f; c->T_east = 500.f;
    c->eps_west = 1.f; c->eps_east = 1.f;
    c->toll = 1.0e-3f;
    c->max_steps = 100000;
    c->grid_num = 1;
    c->model = DNSMC_MODEL_PARTICLE;
    c->kappa = 1.0f;
    c->n_groups = 1;
    c->seed = 1234;
    c->sampler = DNSMC_SAMPLER_IID;
    c->local_sampling = 0;
    c->control_variate = 0;
    c->cv_moments = 0;
    c->block_threads = 0;
    c->tile_a = 0;
    c->mg_steps = 5;  // code/param.h:18-37 (maxs of every grid but the last)
}

int dnsmc_config_from_env(dnsmc_config *c) {
    if (!c) return fail(DNSMC_ERR_ARG, "null config");
    struct { const char *name; int *iv; float *fv; } items[] = {
        {"DNSMC_IMAX", &c->imax, nullptr}, {"DNSMC_JMAX", &c->jmax, nullptr}, {"DNSMC_KMAX", &c->kmax, nullptr},
        {"DNSMC_PROW", &c->p_row, nullptr}, {"DNSMC_NVAR", &c->nvar, nullptr}, {"DNSMC_PHOTMAX", &c->photmax, nullptr},
        {"DNSMC_MODEL", &c->model, nullptr}, {"DNSMC_GRID_NUM", &c->grid_num, nullptr},
        {"DNSMC_MG_STEPS", &c->mg_steps, nullptr},
        {"DNSMC_STRETCHED", &c->stretched_x, nullptr}, {"DNSMC_GROUPS", &c->n_groups, nullptr},
        {"DNSMC_LX", nullptr, &c->Lx}, {"DNSMC_LY", nullptr, &c->Ly}, {"DNSMC_LZ", nullptr, &c->Lz},
        {"DNSMC_TWEST", nullptr, &c->T_west}, {"DNSMC_TEAST", nullptr, &c->T_east},
        {"DNSMC_KAPPA", nullptr, &c->kappa},
    };
    for (auto &it : items) {
        const char *v = getenv(it.name);
        if (!v || !*v) continue;
        char *end = nullptr;
        if (it.iv) {
            long x = strtol(v, &end, 10);
            if (*end) return fail(DNSMC_ERR_ARG, "%s=%s is not an integer", it.name, v);
            *it.iv = (int)x;
        } else {
            float x = strtof(v, &end);
            if (*end) return fail(DNSMC_ERR_ARG, "%s=%s is not a number", it.name, v);
            *it.fv = x;
        }
    }
    const char *sd = getenv("DNSMC_SEED");
    if (sd && *sd) {
        char *end = nullptr;
        unsigned long long x = strtoull(sd, &end, 10);
        if (*end) return fail(DNSMC_ERR_ARG, "DNSMC_SEED=%s is not an integer", sd);
        c->seed = x;
    }
    return DNSMC_OK;
}

int dnsmc_create(const dnsmc_config *cfg, dnsmc_solver **out) {
    if (!cfg || !out) return fail(DNSMC_ERR_ARG, "null argument");
    *out = nullptr;
    TRY(check_config(*cfg));
    dnsmc_solver *s = new dnsmc_solver();
    s->cfg = *cfg;
    make_faces(cfg->imax, cfg->Lx, cfg->stretched_x, s->fw);
    s->da = cfg->Ly / (float)cfg->jmax;
    s->db = cfg->Lz / (float)cfg->kmax;
    s->r_i0 = 0; s->r_i1 = cfg->imax; s->r_j0 = 0; s->r_j1 = cfg->jmax; s->r_k0 = 0; s->r_k1 = cfg->kmax;
    s->rays = cfg->nvar * cfg->photmax;  // a multiple of nvar
    if (cfg->model == DNSMC_MODEL_GREY) s->tab.valid = true;
    *out = s;
    return DNSMC_OK;
}

int dnsmc_destroy(dnsmc_solver *s) {
    if (!s) return DNSMC_OK;
    if (!s->dev_ready) { delete s; return DNSMC_OK; }
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
    s->d_fw.release(); s->d_k.release(); s->d_ib.release(); s->d_ibw.release();
    s->d_slab.release(); s->d_posT.release(); s->d_posTX.release();
    s->d_cv_grp.release(); s->d_cv_sid.release(); s->d_cv_C.release(); s->d_layer.release();
    s->d_sur.release(); s->d_surtab.release(); s->d_Jhat.release(); s->d_Jf.release(); s->d_cv_Cf.release(); s->d_muY.release(); s->d_cvnodes.release(); s->d_beta.release(); s->d_moments.release();
    s->d_fieldT.release(); s->d_fieldTX.release(); s->d_raw.release();
    s->d_stat_part.release(); s->d_stat_out.release(); s->d_rays_pp.release(); s->d_rays_rcp.release(); s->d_item_steps.release(); s->d_kP.release();
    s->d_order.release(); s->d_order_hist.release();
    s->d_mgT.release(); s->d_mgfw.release(); s->d_mgpos.release(); s->d_mgtmp.release();
    s->d_part.release(); s->d_fieldV.release(); s->d_layerV.release();
    s->d_entries.release(); s->d_group_start.release(); s->d_group_empty.release();
    s->d_tally.release(); s->d_Q.release(); s->d_var.release(); s->d_sig.release(); s->h_sig.release(); s->d_Qg.release(); s->d_varg.release();
    s->h_Q.release(); s->d_misc.release(); s->d_counters.release();
    s->d_Qf.release(); s->d_sigf.release(); s->h_Qf.release(); s->h_sigf.release();
    if (s->ev_march0) cudaEventDestroy(s->ev_march0);
    if (s->ev_march1) cudaEventDestroy(s->ev_march1);
    if (s->ev_done) cudaEventDestroy(s->ev_done);
    if (s->ev_solve0) cudaEventDestroy(s->ev_solve0);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return DNSMC_OK;
}

int dnsmc_load_tables_ref(dnsmc_solver *s, const char *dir, int model, int nT, int nB, int nQ) {
    if (!s || !dir) return fail(DNSMC_ERR_ARG, "null argument");
    if (nT < 2 || nB < 1 || nQ < 1) return fail(DNSMC_ERR_ARG, "bad table sizes");
    HostTable t;
    if (model == DNSMC_MODEL_CK) {
        TRY(read_ck_tables(dir, nT, nB, nQ, t));
    } else if (model == DNSMC_MODEL_PARTICLE) {
        TRY(read_particle_tables(dir, nT, nB, t));
    } else {
        return fail(DNSMC_ERR_ARG, "dnsmc_load_tables_ref: model must be CK (0) or PARTICLE (2)");
    }
    if (!(t.dT > 0)) return fail(DNSMC_ERR_TABLE, "table temperatures are not increasing");
    t.valid = true;
    s->tab = std::move(t);
    s->tables_dirty = true;
    return DNSMC_OK;
}

int dnsmc_use_grey_band_tables(dnsmc_solver *s, int nB, int nT, float wvmax, float Tmin) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    if (nB < 1 || nT < 2 || !(wvmax > 0) || !(Tmin > 0)) return fail(DNSMC_ERR_ARG, "bad grey-band parameters");
    HostTable t;
    t.grey_bands = true;
    t.gb_nB = nB; t.gb_nT = nT; t.gb_wvmax = wvmax; t.gb_Tmin = Tmin; t.gb_kappa = s->cfg.kappa;
    s->tab = std::move(t);
    s->tables_dirty = true;
    return DNSMC_OK;
}

int dnsmc_set_table(dnsmc_solver *s, const dnsmc_table_desc *d) {
    if (!s || !d) return fail(DNSMC_ERR_ARG, "null argument");
    if (d->nbands < 1 || d->nq < 1 || d->nT < 2 || d->nX < 1 || !d->k || !d->wvc)
        return fail(DNSMC_ERR_ARG, "bad table description");
    if (d->nbands > 65535) return fail(DNSMC_ERR_ARG, "at most 65535 bands");
    if (!(d->dT > 0) || (d->nX > 1 && !(d->dX > 0))) return fail(DNSMC_ERR_ARG, "table grid steps must be > 0");
    if (!d->prob && (!d->dnu || !d->wq)) return fail(DNSMC_ERR_ARG, "dnu and wq are needed without reference CDFs");
    if (d->prob && !d->kP) return fail(DNSMC_ERR_ARG, "reference sampling needs kP");
    HostTable t;
    t.nbands = d->nbands; t.nq = d->nq; t.nT = d->nT; t.nX = d->nX;
    t.T0 = d->T0; t.dT = d->dT; t.X0 = d->X0; t.dX = d->nX > 1 ? d->dX : 1.0f;
    const size_t nk = (size_t)t.nbands * t.nq * t.nT * t.nX;
    t.k.assign(d->k, d->k + nk);
    for (float v : t.k)
        if (!(v >= 0) || !std::isfinite(v)) return fail(DNSMC_ERR_TABLE, "absorption coefficients must be finite and >= 0");
    t.wvc.assign(d->wvc, d->wvc + t.nbands);
    if (d->dnu) t.dnu.assign(d->dnu, d->dnu + t.nbands); else t.dnu.assign(t.nbands, 0.f);
    if (d->wq) t.wq.assign(d->wq, d->wq + t.nq); else t.wq.assign(t.nq, 1.0f / t.nq);
    if (d->Ib) t.Ib.assign(d->Ib, d->Ib + (size_t)t.nbands * t.nT);
    if (d->prob) {
        t.prob.assign(d->prob, d->prob + (size_t)t.nT * t.nbands);
        if (d->probg) t.probg.assign(d->probg, d->probg + (size_t)t.nT * t.nbands * t.nq);
        t.kP.assign(d->kP, d->kP + t.nT);
        t.ref_sampling = true;
    }
    t.valid = true;
    s->tab = std::move(t);
    s->tables_dirty = true;
    return DNSMC_OK;
}

// ---- binary table file (no counterpart in the reference) -------------------
// The reference reads its tables from text every call (code/read_tables.cpp,
// written by distr/write_tables.cpp:23-107) and has no x_H2O axis.  This
// file holds the whole k(band, g, T, x) table once, little-endian:
//   72-byte header: magic "DNSMCKT1", u32 version (1), u32 header bytes (72),
//   i32 nbands, nq, nT, nX, f32 T0, dT, X0, dX, u32 flags (1: Ib, 2: the
//   reference CDFs prob and kP, 4: the g CDF probg), u32 0, u64 payload
//   bytes, u64 FNV-1a hash of the payload;
//   payload, float32: k[nbands][nq][nT][nX], wvc[nbands], dnu[nbands],
//   wq[nq], then Ib[nbands][nT], prob[nT][nbands] and kP[nT],
//   probg[nT][nbands][nq] as flagged.
namespace {
constexpr char kTabMagic[8] = {'D', 'N', 'S', 'M', 'C', 'K', 'T', '1'};
constexpr uint32_t kTabHeader = 72;

uint64_t fnv1a(const unsigned char *p, size_t n, uint64_t h = 0xcbf29ce484222325ull) {
    for (size_t i = 0; i < n; ++i) { h ^= p[i]; h *= 0x100000001b3ull; }
    return h;
}
void put_u32(std::vector<unsigned char> &b, uint32_t v) { for (int i = 0; i < 4; ++i) b.push_back((unsigned char)(v >> (8 * i))); }
void put_u64(std::vector<unsigned char> &b, uint64_t v) { for (int i = 0; i < 8; ++i) b.push_back((unsigned char)(v >> (8 * i))); }
void put_f32(std::vector<unsigned char> &b, float f) { uint32_t v; memcpy(&v, &f, 4); put_u32(b, v); }
uint32_t get_u32(const unsigned char *p) { return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24; }
uint64_t get_u64(const unsigned char *p) { return (uint64_t)get_u32(p) | (uint64_t)get_u32(p + 4) << 32; }
float get_f32(const unsigned char *p) { const uint32_t v = get_u32(p); float f; memcpy(&f, &v, 4); return f; }
}  // namespace

int dnsmc_save_table(const dnsmc_solver *s, const char *path) {
    if (!s || !path) return fail(DNSMC_ERR_ARG, "null argument");
    if (s->tab.grey_bands) return fail(DNSMC_ERR_STATE, "the reference grey tables are rebuilt at every solve");
    if (!s->tab.valid) return fail(DNSMC_ERR_STATE, "no table to save");
    const HostTable &t = s->tab;
    const uint32_t flags = (t.Ib.empty() ? 0u : 1u) | (t.ref_sampling ? 2u : 0u) | (t.probg.empty() ? 0u : 4u);
    std::vector<unsigned char> pay;
    auto arr = [&](const std::vector<float> &v) { for (float f : v) put_f32(pay, f); };
    arr(t.k); arr(t.wvc); arr(t.dnu); arr(t.wq);
    if (flags & 1u) arr(t.Ib);
    if (flags & 2u) { arr(t.prob); arr(t.kP); }
    if (flags & 4u) arr(t.probg);
    std::vector<unsigned char> h(kTabMagic, kTabMagic + 8);
    put_u32(h, 1); put_u32(h, kTabHeader);
    put_u32(h, (uint32_t)t.nbands); put_u32(h, (uint32_t)t.nq); put_u32(h, (uint32_t)t.nT); put_u32(h, (uint32_t)t.nX);
    put_f32(h, t.T0); put_f32(h, t.dT); put_f32(h, t.X0); put_f32(h, t.dX);
    put_u32(h, flags); put_u32(h, 0);
    put_u64(h, (uint64_t)pay.size()); put_u64(h, fnv1a(pay.data(), pay.size()));
    FILE *f = fopen(path, "wb");
    if (!f) return fail(DNSMC_ERR_IO, "cannot open %s for writing", path);
    const bool ok = fwrite(h.data(), 1, h.size(), f) == h.size() && fwrite(pay.data(), 1, pay.size(), f) == pay.size();
    if (fclose(f) != 0 || !ok) return fail(DNSMC_ERR_IO, "short write to %s", path);
    return DNSMC_OK;
}

int dnsmc_load_table(dnsmc_solver *s, const char *path) {
    if (!s || !path) return fail(DNSMC_ERR_ARG, "null argument");
    FILE *f = fopen(path, "rb");
    if (!f) return fail(DNSMC_ERR_IO, "cannot open %s", path);
    unsigned char h[kTabHeader];
    if (fread(h, 1, kTabHeader, f) != kTabHeader) { fclose(f); return fail(DNSMC_ERR_IO, "%s: short header", path); }
    if (memcmp(h, kTabMagic, 8) != 0) { fclose(f); return fail(DNSMC_ERR_IO, "%s: not a dnsmc table file", path); }
    if (get_u32(h + 8) != 1 || get_u32(h + 12) != kTabHeader) {
        fclose(f);
        return fail(DNSMC_ERR_IO, "%s: unsupported table file version", path);
    }
    const int nb = (int)get_u32(h + 16), nq = (int)get_u32(h + 20), nT = (int)get_u32(h + 24), nX = (int)get_u32(h + 28);
    const uint32_t flags = get_u32(h + 48);
    const uint64_t nbytes = get_u64(h + 56), hash = get_u64(h + 64);
    if (nb < 1 || nq < 1 || nT < 2 || nX < 1 || nb > 65535 || nq > 4096 || nT > 1000000 || nX > 1000000 || (flags & ~7u)) {
        fclose(f);
        return fail(DNSMC_ERR_IO, "%s: bad table sizes in the header", path);
    }
    const uint64_t nk = (uint64_t)nb * nq * nT * nX;
    uint64_t nf = nk + 2ull * nb + nq;
    if (flags & 1u) nf += (uint64_t)nb * nT;
    if (flags & 2u) nf += (uint64_t)nT * nb + nT;
    if (flags & 4u) nf += (uint64_t)nT * nb * nq;
    if (nbytes != 4 * nf || nf > (1ull << 32)) { fclose(f); return fail(DNSMC_ERR_IO, "%s: payload size does not match the header", path); }
    std::vector<unsigned char> pay((size_t)nbytes);
    const size_t got = fread(pay.data(), 1, pay.size(), f);
    const bool extra = fgetc(f) != EOF;
    fclose(f);
    if (got != pay.size() || extra) return fail(DNSMC_ERR_IO, "%s: payload length differs from the header", path);
    if (fnv1a(pay.data(), pay.size()) != hash) return fail(DNSMC_ERR_IO, "%s: payload checksum mismatch", path);
    std::vector<float> v((size_t)nf);
    for (size_t i = 0; i < v.size(); ++i) v[i] = get_f32(pay.data() + 4 * i);
    const float *p = v.data();
    dnsmc_table_desc d{};
    d.nbands = nb; d.nq = nq; d.nT = nT; d.nX = nX;
    d.T0 = get_f32(h + 32); d.dT = get_f32(h + 36); d.X0 = get_f32(h + 40); d.dX = get_f32(h + 44);
    d.k = p; p += nk;
    d.wvc = p; p += nb;
    d.dnu = p; p += nb;
    d.wq = p; p += nq;
    if (flags & 1u) { d.Ib = p; p += (size_t)nb * nT; }
    if (flags & 2u) { d.prob = p; p += (size_t)nT * nb; d.kP = p; p += nT; }
    if (flags & 4u) { d.probg = p; p += (size_t)nT * nb * nq; }
    return dnsmc_set_table(s, &d);
}

int dnsmc_get_table_info(const dnsmc_solver *s, int *nbands, int *nq, int *nT, int *nX, float *T0, float *dT,
                         float *X0, float *dX) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    const HostTable &t = s->tab;
    if (nbands) *nbands = t.nbands;
    if (nq) *nq = t.nq;
    if (nT) *nT = t.nT;
    if (nX) *nX = t.nX;
    if (T0) *T0 = t.T0;
    if (dT) *dT = t.dT;
    if (X0) *X0 = t.X0;
    if (dX) *dX = t.dX;
    return DNSMC_OK;
}

int dnsmc_get_table(const dnsmc_solver *s, float *k, float *wvc, float *Ib, float *prob, float *probg, float *kP) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    HostTable t = s->tab;
    fill_ib(t);
    if (k) std::copy(t.k.begin(), t.k.end(), k);
    if (wvc) std::copy(t.wvc.begin(), t.wvc.end(), wvc);
    if (Ib) std::copy(t.Ib.begin(), t.Ib.end(), Ib);
    if (prob) std::copy(t.prob.begin(), t.prob.end(), prob);
    if (probg) std::copy(t.probg.begin(), t.probg.end(), probg);
    if (kP) std::copy(t.kP.begin(), t.kP.end(), kP);
    return DNSMC_OK;
}

int dnsmc_prepare_sampling(dnsmc_solver *s, float Tmax, float xmean) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    if (!(Tmax > 0)) return fail(DNSMC_ERR_ARG, "Tmax must be > 0");
    if (s->cfg.model != DNSMC_MODEL_GREY && !s->tab.valid && !s->tab.grey_bands)
        return fail(DNSMC_ERR_STATE, "no tables: load or set tables first");
    if (s->tab.grey_bands) { build_grey_band_tables(s->tab, Tmax); s->tables_dirty = true; }
    s->tmax_used = Tmax;
    s->sampling_valid = false;  // the host tables now differ from the device's: the next solve rebuilds
    return build_sampling(s, Tmax, xmean);
}

int dnsmc_set_fields(dnsmc_solver *s, int nfields, const float *T, const float *x, int layout) {
    if (!s || !T || nfields < 1) return fail(DNSMC_ERR_ARG, "bad arguments");
    if (nfields > 65535) return fail(DNSMC_ERR_ARG, "at most 65535 fields per solve");
    return upload_fields_host(s, nfields, T, x, layout);
}

int dnsmc_set_fields_device(dnsmc_solver *s, int nfields, const float *dT, const float *dx) {
    if (!s || !dT || nfields < 1) return fail(DNSMC_ERR_ARG, "bad arguments");
    if (nfields > 65535) return fail(DNSMC_ERR_ARG, "at most 65535 fields per solve");
    const dnsmc_config &c = s->cfg;
    const long long ncell = (long long)c.imax * c.jmax * c.kmax;
    TRY(set_device(s));
    TRY(wait_done(s, 0));
    if (dx) TRY(s->d_fieldTX.ensure((size_t)nfields * ncell));
    else TRY(s->d_fieldT.ensure((size_t)nfields * ncell));
    for (int f = 0; f < nfields; ++f) {
        int rc;
        if (dx)
            rc = launch_pack_TX(dT + f * ncell, dx + f * ncell, s->d_fieldTX.p + f * ncell, c.imax, c.jmax, c.kmax, 1, c.imax, (long long)c.imax * c.jmax, 0, s->stream);
        else
            rc = launch_pack_T(dT + f * ncell, s->d_fieldT.p + f * ncell, c.imax, c.jmax, c.kmax, 1, c.imax, (long long)c.imax * c.jmax, 0, s->stream);
        if (rc) return fail(DNSMC_ERR_CUDA, "pack launch: %s", cudaGetErrorString((cudaError_t)rc));
    }
    double st[4];
    TRY(field_stats_checked(s, nfields, dx != nullptr, st));
    if (c.grid_num > 1)
        TRY(upload_coarse(s, nfields, dx ? (const float *)s->d_fieldTX.p : s->d_fieldT.p, dx ? 2 : 1));
    s->nfields = nfields;
    s->have_x = dx != nullptr;
    s->tmax_fields = (float)st[0];
    s->tmin_fields = (float)st[1];
    s->xsum = st[2];
    return DNSMC_OK;
}

int dnsmc_set_particles(dnsmc_solver *s, int nbands, const float *absorption, const float *scattering, float hg_g) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    TRY(wait_done(s, 0));
    if (!absorption && !scattering) {
        s->part.clear();
        s->fv_fields = 0;
        return DNSMC_OK;
    }
    const dnsmc_config &c = s->cfg;
    if (c.model != DNSMC_MODEL_GREY && c.model != DNSMC_MODEL_TABLE)
        return fail(DNSMC_ERR_ARG, "particles need the grey model or raw k tables (dnsmc_set_table)");
    const int nb = c.model == DNSMC_MODEL_GREY ? 1 : s->tab.nbands;
    if (c.model == DNSMC_MODEL_TABLE && !s->tab.valid) return fail(DNSMC_ERR_STATE, "set the k table before the particles");
    if (nbands != nb) return fail(DNSMC_ERR_ARG, "particle table has %d bands, the spectral model %d", nbands, nb);
    if (!(hg_g > -1.0f && hg_g < 1.0f)) return fail(DNSMC_ERR_ARG, "Henyey-Greenstein g must be in (-1, 1)");
    std::vector<float2> pp((size_t)nb);
    for (int b = 0; b < nb; ++b) {
        const float a = absorption ? absorption[b] : 0.0f, sc = scattering ? scattering[b] : 0.0f;
        if (!(a >= 0.0f) || !(sc >= 0.0f) || !std::isfinite(a) || !std::isfinite(sc))
            return fail(DNSMC_ERR_ARG, "particle coefficients must be finite and >= 0");
        pp[(size_t)b] = make_float2(a, sc);
    }
    TRY(set_device(s));
    TRY(s->d_part.ensure(pp.size()));
    CUDA_TRY(cudaMemcpy(s->d_part.p, pp.data(), pp.size() * sizeof(float2), cudaMemcpyHostToDevice));
    s->part = pp;
    s->hg_g = hg_g;
    return DNSMC_OK;
}

int dnsmc_set_particle_field(dnsmc_solver *s, const float *fv, int layout) {
    if (!s || !fv) return fail(DNSMC_ERR_ARG, "null argument");
    if (s->nfields < 1) return fail(DNSMC_ERR_STATE, "set the temperature fields first");
    const dnsmc_config &c = s->cfg;
    const long long ncell = (long long)c.imax * c.jmax * c.kmax;
    long long sj, sk, base, nsrc;
    if (layout == DNSMC_LAYOUT_DENSE) {
        sj = c.imax; sk = (long long)c.imax * c.jmax; base = 0; nsrc = ncell;
    } else if (layout == DNSMC_LAYOUT_FORTRAN) {
        sj = c.imax + 2; sk = (long long)(c.imax + 2) * (c.jmax + 2);
        base = 1 + sj + sk;
        nsrc = (long long)(c.imax + 2) * (c.jmax + 2) * (c.kmax + 2);
    } else {
        return fail(DNSMC_ERR_ARG, "unknown layout %d", layout);
    }
    float vmax = 0.0f;
    double vsum = 0.0;
    for (int f = 0; f < s->nfields; ++f)
        for (int k = 0; k < c.kmax; ++k)
            for (int j = 0; j < c.jmax; ++j) {
                const long long o = f * nsrc + base + j * sj + k * sk;
                for (int i = 0; i < c.imax; ++i) {
                    const float v = fv[o + i];
                    if (!(v >= 0.0f) || !std::isfinite(v)) return fail(DNSMC_ERR_ARG, "volume fractions must be finite and >= 0");
                    vmax = std::max(vmax, v);
                    vsum += v;
                }
            }
    TRY(set_device(s));
    TRY(wait_done(s, 0));
    TRY(s->d_raw.ensure((size_t)nsrc));
    TRY(s->d_fieldV.ensure((size_t)s->nfields * ncell));
    for (int f = 0; f < s->nfields; ++f) {
        CUDA_TRY(cudaMemcpyAsync(s->d_raw.p, fv + f * nsrc, nsrc * sizeof(float), cudaMemcpyHostToDevice, s->stream));
        const int rc = launch_pack_T(s->d_raw.p, s->d_fieldV.p + f * ncell, c.imax, c.jmax, c.kmax, 1, sj, sk, base,
                                     s->stream);
        if (rc) return fail(DNSMC_ERR_CUDA, "pack launch: %s", cudaGetErrorString((cudaError_t)rc));
    }
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->fv_fields = s->nfields;
    s->fv_max = vmax;
    s->fv_mean = vsum / ((double)s->nfields * ncell);
    return DNSMC_OK;
}

int dnsmc_set_region(dnsmc_solver *s, int i0, int i1, int j0, int j1, int k0, int k1) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    const dnsmc_config &c = s->cfg;
    if (i0 < 0 || i1 > c.imax || i0 >= i1 || j0 < 0 || j1 > c.jmax || j0 >= j1 || k0 < 0 || k1 > c.kmax || k0 >= k1)
        return fail(DNSMC_ERR_ARG, "region out of range");
    TRY(wait_done(s, 0));
    s->r_i0 = i0; s->r_i1 = i1; s->r_j0 = j0; s->r_j1 = j1; s->r_k0 = k0; s->r_k1 = k1;
    s->rays_pp.clear();
    s->rays_pg = 0;
    s->rays_dev = false;
    return DNSMC_OK;
}

int dnsmc_packet_shape(const dnsmc_solver *s, int *tile_a, int *tile_b) {
    if (!s || !tile_a || !tile_b) return fail(DNSMC_ERR_ARG, "null argument");
    int npa, npb, npw;
    tiling(s, tile_a, tile_b, &npa, &npb, &npw);
    return DNSMC_OK;
}

int dnsmc_packet_count(const dnsmc_solver *s, int *npackets) {
    if (!s || !npackets) return fail(DNSMC_ERR_ARG, "null argument");
    int ta, tb, npa, npb, npw;
    tiling(s, &ta, &tb, &npa, &npb, &npw);
    *npackets = npa * npb * npw;
    return DNSMC_OK;
}

int dnsmc_set_rays(dnsmc_solver *s, int rays_per_group, const int *rays_per_packet) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    if (rays_per_group < 1 && !rays_per_packet) return fail(DNSMC_ERR_ARG, "rays must be >= 1");
    const int B = s->cfg.sampler == DNSMC_SAMPLER_RQMC ? s->cfg.nvar : 1;
    if (!rays_per_packet && rays_per_group % B)
        return fail(DNSMC_ERR_ARG, "RQMC: rays per group (%d) must be a multiple of nvar (%d)", rays_per_group, B);
    TRY(wait_done(s, 0));
    s->rays = rays_per_group;
    if (rays_per_packet) {
        TRY(set_device(s));
        int np;
        TRY(dnsmc_packet_count(s, &np));
        for (int i = 0; i < np; ++i) {
            if (rays_per_packet[i] < 0) return fail(DNSMC_ERR_ARG, "negative ray count");
            if (rays_per_packet[i] % B) return fail(DNSMC_ERR_ARG, "RQMC: per-packet rays must be multiples of nvar");
        }
        s->rays_pp.assign(rays_per_packet, rays_per_packet + np);
        s->rays_np = np;
        TRY(s->d_rays_pp.ensure(np));
        CUDA_TRY(cudaMemcpy(s->d_rays_pp.p, s->rays_pp.data(), np * sizeof(int), cudaMemcpyHostToDevice));
    } else {
        s->rays_pp.clear();
    }
    s->rays_pg = 0;
    s->rays_dev = false;
    return DNSMC_OK;
}

int dnsmc_set_rays_per_item(dnsmc_solver *s, int n_groups, const int *rays) {
    if (!s || !rays) return fail(DNSMC_ERR_ARG, "null argument");
    if (n_groups < 1) return fail(DNSMC_ERR_ARG, "n_groups must be >= 1");
    const int B = s->cfg.sampler == DNSMC_SAMPLER_RQMC ? s->cfg.nvar : 1;
    int np;
    TRY(dnsmc_packet_count(s, &np));
    const size_t n = (size_t)n_groups * np;
    for (size_t i = 0; i < n; ++i) {
        if (rays[i] < 0) return fail(DNSMC_ERR_ARG, "negative ray count");
        if (rays[i] % B) return fail(DNSMC_ERR_ARG, "RQMC: per-item rays must be multiples of nvar");
    }
    TRY(set_device(s));
    TRY(wait_done(s, 0));
    s->rays_pp.assign(rays, rays + n);
    s->rays_pg = n_groups;
    s->rays_dev = false;
    s->rays_np = np;
    TRY(s->d_rays_pp.ensure(n));
    CUDA_TRY(cudaMemcpy(s->d_rays_pp.p, s->rays_pp.data(), n * sizeof(int), cudaMemcpyHostToDevice));
    return DNSMC_OK;
}

int dnsmc_get_coarse_field(dnsmc_solver *s, int field, int level, float *T) {
    if (!s || !T) return fail(DNSMC_ERR_ARG, "null argument");
    const dnsmc_config &c = s->cfg;
    if (level < 1 || level >= c.grid_num) return fail(DNSMC_ERR_ARG, "level must be 1..grid_num-1");
    if (field < 0 || field >= s->mg_fields) return fail(DNSMC_ERR_ARG, "no such field");
    TRY(set_device(s));
    TRY(wait_done(s, 0));
    const int im = c.imax >> level, jm = c.jmax >> level, km = c.kmax >> level;
    const size_t n = (size_t)im * jm * km;
    std::vector<float> h(n);
    CUDA_TRY(cudaStreamSynchronize(s->stream));  // the coarsening runs on the solver's stream
    CUDA_TRY(cudaMemcpy(h.data(), s->d_mgT.p + s->mg_off[level] + (long long)field * n, n * sizeof(float),
                        cudaMemcpyDeviceToHost));
    for (int i = 0; i < im; ++i)
        for (int k = 0; k < km; ++k)
            for (int j = 0; j < jm; ++j) T[(size_t)i + (size_t)im * (j + (size_t)jm * k)] = h[((size_t)i * km + k) * jm + j];
    return DNSMC_OK;
}

int dnsmc_set_graph(dnsmc_solver *s, int enable) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    TRY(wait_done(s, 0));
    s->graph_on = enable != 0;
    if (!s->graph_on && s->graph_exec) {
        TRY(set_device(s));
        cudaGraphExecDestroy(s->graph_exec);
        s->graph_exec = nullptr;
        s->graph_key.clear();
    }
    return DNSMC_OK;
}

int dnsmc_get_launch_count(long long *n) {
    if (!n) return fail(DNSMC_ERR_ARG, "null argument");
    *n = launch_count();
    return DNSMC_OK;
}

int dnsmc_get_graph_info(const dnsmc_solver *s, long long *captures, long long *launches) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    if (captures) *captures = s->graph_captures;
    if (launches) *launches = s->graph_launches;
    return DNSMC_OK;
}

int dnsmc_set_rays_adaptive(dnsmc_solver *s, float rays_per_tau, int min_rays, int max_rays) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    const dnsmc_config &c = s->cfg;
    const int B = c.sampler == DNSMC_SAMPLER_RQMC ? c.nvar : 1;
    if (!(rays_per_tau > 0) || min_rays < std::max(2, B) || max_rays < min_rays || min_rays % B || max_rays % B)
        return fail(DNSMC_ERR_ARG, "need rays_per_tau > 0 and max(2, nvar) <= min_rays <= max_rays, multiples of nvar");
    if (s->nfields < 1) return fail(DNSMC_ERR_STATE, "no fields: call dnsmc_set_fields first");
    if (c.model != DNSMC_MODEL_GREY && !s->tab.valid && !s->tab.grey_bands)
        return fail(DNSMC_ERR_STATE, "no tables: load or set tables first");
    TRY(set_device(s));
    TRY(wait_done(s, 0));
    AdaptParams A;
    memset(&A, 0, sizeof A);
    const HostTable &t = s->tab;
    int mode = MODE_GREY;
    if (c.model != DNSMC_MODEL_GREY) {
        if (s->tab.grey_bands) {
            const float Tmax = std::max(s->tmax_fields, std::max(c.T_west, c.T_east));
            build_grey_band_tables(s->tab, Tmax);
            s->tables_dirty = true;
        }
        if (s->tables_dirty) TRY(upload_tables(s));
        mode = t.nX > 1 ? MODE_TX : MODE_T;
        // Planck-mean absorption coefficient on the table grid:
        // kP(T, x) = pi sum_b sum_g w_g k_bg(T, x) Ib_b(T) dnu_b / (sigma T^4)
        std::vector<float> kp((size_t)t.nT * t.nX);
        const int nq = std::max(1, t.nq);
        for (int ti = 0; ti < t.nT; ++ti) {
            const double T = t.T0 + ti * (double)t.dT;
            const double den = kSigma * T * T * T * T;
            for (int xi = 0; xi < t.nX; ++xi) {
                double acc = 0.0;
                for (int b = 0; b < t.nbands; ++b) {
                    const double ib = t.Ib[(size_t)b * t.nT + ti] * (double)t.dnu[b] * 100.0;
                    const float *kb = t.k.data() + (size_t)b * nq * t.nT * t.nX;
                    for (int g = 0; g < nq; ++g)
                        acc += (double)(t.wq.empty() ? 1.0f : t.wq[g]) *
                               kb[((size_t)g * t.nT + ti) * t.nX + xi] * ib;
                }
                kp[(size_t)ti * t.nX + xi] = den > 0 ? (float)(kPi * acc / den) : 0.0f;
            }
        }
        TRY(s->d_kP.ensure(kp.size()));
        CUDA_TRY(cudaMemcpyAsync(s->d_kP.p, kp.data(), kp.size() * sizeof(float), cudaMemcpyHostToDevice, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        A.kP = s->d_kP.p;
        A.nT = t.nT; A.nX = t.nX;
        A.T0 = t.T0; A.invdT = 1.0f / t.dT; A.X0 = t.X0; A.invdX = 1.0f / t.dX;
    }
    int ni, nj, nk, ta, tb, npa, npb, npw;
    region_dims(s, &ni, &nj, &nk);
    tiling(s, &ta, &tb, &npa, &npb, &npw);
    const int np = npa * npb * npw;
    TRY(s->d_rays_pp.ensure((size_t)np));
    A.nfields = s->nfields; A.nw = c.imax; A.na = c.jmax; A.nb = c.kmax; A.mode = mode;
    A.fT = s->d_fieldT.p; A.fTX = s->d_fieldTX.p; A.fw = s->d_fw.p; A.da = s->da; A.db = s->db;
    A.ew0 = s->r_i0; A.ea0 = s->r_j0; A.eb0 = s->r_k0; A.njR = nj; A.nkR = nk;
    A.tile_a = ta; A.tile_b = tb; A.npa = npa; A.npb = npb; A.n_packets = np;
    A.field_stride = (long long)c.imax * c.jmax * c.kmax;
    A.kappa = c.kappa;
    A.per_tau = rays_per_tau; A.B = B; A.nmin = min_rays; A.nmax = max_rays;
    A.rays = s->d_rays_pp.p;
    const int rc = launch_adaptive_rays(A, s->stream);
    if (rc) return fail(DNSMC_ERR_CUDA, "adaptive rays launch: %s", cudaGetErrorString((cudaError_t)rc));
    s->rays_pp.clear();
    s->rays_pg = 0;
    s->rays_dev = true;
    s->rays_np = np;
    return DNSMC_OK;
}

int dnsmc_get_stream(dnsmc_solver *s, void **stream) {
    if (!s || !stream) return fail(DNSMC_ERR_ARG, "null argument");
    TRY(set_device(s));
    *stream = (void *)s->stream;
    return DNSMC_OK;
}

int dnsmc_get_rays_per_item(dnsmc_solver *s, int *n_groups, int *rays) {
    if (!s || !n_groups) return fail(DNSMC_ERR_ARG, "null argument");
    TRY(wait_done(s, 0));
    // -1: one row of per-packet counts shared by all band groups
    *n_groups = (s->rays_pp.empty() && !s->rays_dev) ? 0 : (s->rays_pg > 0 ? s->rays_pg : -1);
    if (!rays || *n_groups == 0) return DNSMC_OK;
    int np;
    TRY(dnsmc_packet_count(s, &np));
    const size_t rows = *n_groups > 0 ? (size_t)*n_groups : 1;
    if (s->rays_dev) {
        TRY(set_device(s));
        CUDA_TRY(cudaMemcpy(rays, s->d_rays_pp.p, rows * np * sizeof(int), cudaMemcpyDeviceToHost));
    } else {
        memcpy(rays, s->rays_pp.data(), rows * np * sizeof(int));
    }
    return DNSMC_OK;
}

int dnsmc_get_item_steps(dnsmc_solver *s, double *steps) {
    if (!s || !steps) return fail(DNSMC_ERR_ARG, "null argument");
    TRY(wait_done(s, 0));
    const long long n = s->last.n_items;
    if (n <= 0 || !s->d_item_steps.p) return fail(DNSMC_ERR_STATE, "no solve yet");
    std::vector<unsigned long long> h((size_t)n);
    CUDA_TRY(cudaMemcpy(h.data(), s->d_item_steps.p, (size_t)n * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    for (long long i = 0; i < n; ++i) steps[i] = (double)h[(size_t)i];
    return DNSMC_OK;
}

int dnsmc_solve_async(dnsmc_solver *s) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    TRY(wait_done(s, 0));
    return solve_enqueue(s, false, 0, 0, 0, 0, 0, nullptr, nullptr, nullptr);
}

int dnsmc_wait(dnsmc_solver *s, double timeout_s) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    return wait_done(s, timeout_s);
}

// Host copy of a large result array on several threads: the caller's array
// is often freshly allocated, and its first-touch page faults dominate a
// single-threaded copy.
static void parallel_copy(void *dst, const void *src, size_t bytes) {
    const size_t chunk = (size_t)2 << 20;
    const unsigned nt = (unsigned)std::min<size_t>(8, (bytes + chunk - 1) / chunk);
    if (nt <= 1) { memcpy(dst, src, bytes); return; }
    std::vector<std::thread> th;
    const size_t per = (bytes / nt + 4095) & ~(size_t)4095;
    for (unsigned t = 0; t < nt; ++t) {
        const size_t o = (size_t)t * per;
        if (o >= bytes) break;
        const size_t len = std::min(per, bytes - o);
        th.emplace_back([=] { memcpy((char *)dst + o, (const char *)src + o, len); });
    }
    for (auto &x : th) x.join();
}

// Rows of imax floats of a dense (imax, jl, kmax) block into the interior
// of a Fortran array (0:imax+1, 0:jl+1, 0:kmax+1), several threads over k.
static void scatter_fortran(float *dst, const float *src, int imax, int jl, int kmax) {
    if (!dst) return;
    const unsigned nt = (unsigned)std::max(1, std::min(8, kmax / 8));
    auto part = [=](int k0, int k1) {
        for (int k = k0; k < k1; ++k)
            for (int j = 0; j < jl; ++j)
                memcpy(dst + 1 + (size_t)(imax + 2) * ((j + 1) + (size_t)(jl + 2) * (k + 1)),
                       src + (size_t)imax * (j + (size_t)jl * k), (size_t)imax * sizeof(float));
    };
    if (nt <= 1) { part(0, kmax); return; }
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t) th.emplace_back(part, (int)(t * kmax / nt), (int)((t + 1) * kmax / nt));
    for (auto &x : th) x.join();
}

int dnsmc_get_results(dnsmc_solver *s, double *Q, double *sigma) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    if (!s->solved) return fail(DNSMC_ERR_STATE, "no solve has been run");
    TRY(wait_done(s, 0));
    if (s->solved_result_type != DNSMC_RESULT_F64)
        return fail(DNSMC_ERR_STATE, "the last solve returned float results: use dnsmc_get_results_float");
    const size_t n = (size_t)s->nfields * s->last.region_cells;
    if (Q) parallel_copy(Q, s->h_Q.p, n * sizeof(double));
    if (sigma) parallel_copy(sigma, s->h_sig.p, n * sizeof(double));
    return DNSMC_OK;
}

int dnsmc_set_result_type(dnsmc_solver *s, int type) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    if (type != DNSMC_RESULT_F64 && type != DNSMC_RESULT_F32) return fail(DNSMC_ERR_ARG, "unknown result type %d", type);
    TRY(wait_done(s, 0));
    s->result_type = type;
    return DNSMC_OK;
}

int dnsmc_get_results_float(dnsmc_solver *s, float *Q, float *sigma) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    if (!s->solved) return fail(DNSMC_ERR_STATE, "no solve has been run");
    TRY(wait_done(s, 0));
    const size_t n = (size_t)s->nfields * s->last.region_cells;
    if (s->solved_result_type == DNSMC_RESULT_F32) {
        if (Q) parallel_copy(Q, s->h_Qf.p, n * sizeof(float));
        if (sigma) parallel_copy(sigma, s->h_sigf.p, n * sizeof(float));
    } else {
        for (size_t i = 0; i < n; ++i) {
            if (Q) Q[i] = (float)s->h_Q.p[i];
            if (sigma) sigma[i] = (float)s->h_sig.p[i];
        }
    }
    return DNSMC_OK;
}

int dnsmc_get_group_results(dnsmc_solver *s, double *Qg, double *varg) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    if (!s->solved) return fail(DNSMC_ERR_STATE, "no solve has been run");
    TRY(wait_done(s, 0));
    TRY(set_device(s));
    const size_t n = (size_t)s->nfields * s->last.region_cells * s->last.n_groups;
    if (Qg) CUDA_TRY(cudaMemcpy(Qg, s->d_Qg.p, n * sizeof(double), cudaMemcpyDeviceToHost));
    if (varg) CUDA_TRY(cudaMemcpy(varg, s->d_varg.p, n * sizeof(double), cudaMemcpyDeviceToHost));
    return DNSMC_OK;
}

int dnsmc_status(dnsmc_solver *s, uint32_t *status) {
    if (!s || !status) return fail(DNSMC_ERR_ARG, "null argument");
    TRY(wait_done(s, 0));
    *status = s->h_status;
    return DNSMC_OK;
}

int dnsmc_get_counters(dnsmc_solver *s, double *rays, double *steps, double *march_ms) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    TRY(wait_done(s, 0));
    if (rays) *rays = (double)s->h_counters[0];
    if (steps) *steps = (double)s->h_counters[1];
    if (march_ms) *march_ms = s->march_ms;
    return DNSMC_OK;
}

int dnsmc_get_timing(dnsmc_solver *s, double *solve_ms, double *march_ms) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    TRY(wait_done(s, 0));
    if (solve_ms) *solve_ms = s->solve_ms;
    if (march_ms) *march_ms = s->march_ms;
    return DNSMC_OK;
}

int dnsmc_get_tmax(const dnsmc_solver *s, float *tmax) {
    if (!s || !tmax) return fail(DNSMC_ERR_ARG, "null argument");
    *tmax = s->tmax_used;
    return DNSMC_OK;
}

int dnsmc_get_sampling(const dnsmc_solver *s, int *n_groups, int *n_tbins, int *group_start, int *n_entries,
                       float *prob, int *alias, int *band, int *gq, float *W, float *ibw) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    if (n_groups) *n_groups = s->n_groups_used;
    if (n_tbins) *n_tbins = s->n_tbins_used;
    if (group_start) std::copy(s->group_start.begin(), s->group_start.end(), group_start);
    if (n_entries) *n_entries = (int)s->entries.size();
    const int nq = std::max(1, s->tab.nq);
    for (size_t i = 0; i < s->entries.size(); ++i) {
        const SpecEntry &e = s->entries[i];
        if (prob) prob[i] = e.prob;
        if (alias) alias[i] = (int)(e.alias_nb & 0xFFFFu);
        if (band) band[i] = (int)(e.alias_nb >> 16);
        if (gq) gq[i] = (int)(e.koff % nq);
        if (W) W[i] = e.W;
    }
    if (ibw) std::copy(s->ibw.begin(), s->ibw.end(), ibw);
    return DNSMC_OK;
}

int dnsmc_set_cv_beta(dnsmc_solver *s, const float *beta) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    TRY(wait_done(s, 0));
    if (!beta) { s->beta_set = false; return DNSMC_OK; }
    if (s->nfields < 1) return fail(DNSMC_ERR_STATE, "set fields before the control-variate coefficients");
    int ni, nj, nk;
    region_dims(s, &ni, &nj, &nk);
    const long long rc_ = (long long)ni * nj * nk;
    const int nG = s->cfg.model == DNSMC_MODEL_GREY ? 1 : std::min(s->cfg.n_groups, std::max(1, s->tab.nbands));
    // dense [f][g][k][j][i][2] -> tally layout [f][g][i][k][j]
    std::vector<float2> tl((size_t)s->nfields * nG * rc_);
    for (long long fg = 0; fg < (long long)s->nfields * nG; ++fg)
        for (int k = 0; k < nk; ++k)
            for (int j = 0; j < nj; ++j)
                for (int i = 0; i < ni; ++i) {
                    const float *b = beta + 2 * (fg * rc_ + i + (long long)ni * (j + (long long)nj * k));
                    if (!std::isfinite(b[0]) || !std::isfinite(b[1]))
                        return fail(DNSMC_ERR_ARG, "control-variate coefficients must be finite");
                    tl[fg * rc_ + ((long long)i * nk + k) * nj + j] = make_float2(b[0], b[1]);
                }
    TRY(set_device(s));
    TRY(s->d_beta.ensure(tl.size()));
    CUDA_TRY(cudaMemcpy(s->d_beta.p, tl.data(), tl.size() * sizeof(float2), cudaMemcpyHostToDevice));
    s->beta_set = true;
    return DNSMC_OK;
}

int dnsmc_get_cv_beta(dnsmc_solver *s, float *beta) {
    if (!s || !beta) return fail(DNSMC_ERR_ARG, "null argument");
    TRY(wait_done(s, 0));
    if (!s->beta_set) return fail(DNSMC_ERR_STATE, "no coefficients set: (1, -1) everywhere");
    int ni, nj, nk;
    region_dims(s, &ni, &nj, &nk);
    const long long rc_ = (long long)ni * nj * nk;
    const int nG = s->cfg.model == DNSMC_MODEL_GREY ? 1 : std::min(s->cfg.n_groups, std::max(1, s->tab.nbands));
    const size_t n = (size_t)s->nfields * nG * rc_;
    if (s->d_beta.n < n) return fail(DNSMC_ERR_STATE, "coefficients were set for another region");
    std::vector<float2> tl(n);
    TRY(set_device(s));
    CUDA_TRY(cudaMemcpy(tl.data(), s->d_beta.p, n * sizeof(float2), cudaMemcpyDeviceToHost));
    for (long long fg = 0; fg < (long long)s->nfields * nG; ++fg)
        for (int i = 0; i < ni; ++i)
            for (int k = 0; k < nk; ++k)
                for (int j = 0; j < nj; ++j) {
                    const float2 v = tl[fg * rc_ + ((long long)i * nk + k) * nj + j];
                    float *b = beta + 2 * (fg * rc_ + i + (long long)ni * (j + (long long)nj * k));
                    b[0] = v.x;
                    b[1] = v.y;
                }
    return DNSMC_OK;
}

static void tally_to_dense(const double *src, double *dst, long long nfg, int ni, int nj, int nk, int width) {
    const long long rc_ = (long long)ni * nj * nk;
    for (long long fg = 0; fg < nfg; ++fg)
        for (int i = 0; i < ni; ++i)
            for (int k = 0; k < nk; ++k)
                for (int j = 0; j < nj; ++j)
                    for (int q = 0; q < width; ++q)
                        dst[width * (fg * rc_ + i + (long long)ni * (j + (long long)nj * k)) + q] =
                            src[width * (fg * rc_ + ((long long)i * nk + k) * nj + j) + q];
}

int dnsmc_get_cv_moments(dnsmc_solver *s, double *moments) {
    if (!s || !moments) return fail(DNSMC_ERR_ARG, "null argument");
    if (!s->solved || !s->cfg.control_variate || !s->cfg.cv_moments)
        return fail(DNSMC_ERR_STATE, "no solve with cv_moments = 1 has been run");
    TRY(wait_done(s, 0));
    TRY(set_device(s));
    int ni, nj, nk;
    region_dims(s, &ni, &nj, &nk);
    const long long nfg = (long long)s->nfields * s->last.n_groups;
    std::vector<double> tl((size_t)(nfg * ni * nj * nk * 9));
    CUDA_TRY(cudaMemcpy(tl.data(), s->d_moments.p, tl.size() * sizeof(double), cudaMemcpyDeviceToHost));
    tally_to_dense(tl.data(), moments, nfg, ni, nj, nk, 9);
    return DNSMC_OK;
}

static_assert(kSurBins == DNSMC_CV_BINS, "surrogate bins of the march and of the interface");

int dnsmc_get_cv_table(dnsmc_solver *s, float *tab) {
    if (!s || !tab) return fail(DNSMC_ERR_ARG, "null argument");
    if (!s->solved || !s->cfg.control_variate) return fail(DNSMC_ERR_STATE, "no control-variate solve has been run");
    TRY(wait_done(s, 0));
    TRY(set_device(s));
    const size_t n = (size_t)s->nfields * s->cv_samples * s->cfg.imax * 2 * kSurBins;
    CUDA_TRY(cudaMemcpy(tab, s->d_surtab.p, n * sizeof(float4), cudaMemcpyDeviceToHost));
    return DNSMC_OK;
}

int dnsmc_get_cv_data(dnsmc_solver *s, int *n_samples, float *layer, float *sur, double *Jhat, double *muY) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    if (!s->solved || !s->cfg.control_variate) return fail(DNSMC_ERR_STATE, "no control-variate solve has been run");
    TRY(wait_done(s, 0));
    TRY(set_device(s));
    const int S = s->cv_samples;
    if (n_samples) *n_samples = S;
    const size_t nl = (size_t)s->nfields * s->cfg.imax, ns = nl * S;
    if (layer) CUDA_TRY(cudaMemcpy(layer, s->d_layer.p, nl * sizeof(float2), cudaMemcpyDeviceToHost));
    if (sur) CUDA_TRY(cudaMemcpy(sur, s->d_sur.p, ns * sizeof(float2), cudaMemcpyDeviceToHost));
    if (Jhat) CUDA_TRY(cudaMemcpy(Jhat, s->d_Jhat.p, ns * sizeof(double2), cudaMemcpyDeviceToHost));
    if (muY) {
        int ni, nj, nk;
        region_dims(s, &ni, &nj, &nk);
        const long long nfg = (long long)s->nfields * s->last.n_groups;
        std::vector<double> tl((size_t)(nfg * ni * nj * nk * 2));
        CUDA_TRY(cudaMemcpy(tl.data(), s->d_muY.p, tl.size() * sizeof(double), cudaMemcpyDeviceToHost));
        tally_to_dense(tl.data(), muY, nfg, ni, nj, nk, 2);
    }
    return DNSMC_OK;
}

int dnsmc_get_geometry(const dnsmc_solver *s, float *xu, float *dy, float *dz) {
    if (!s) return fail(DNSMC_ERR_ARG, "null solver");
    if (xu) std::copy(s->fw.begin(), s->fw.end(), xu);
    if (dy) *dy = s->da;
    if (dz) *dz = s->db;
    return DNSMC_OK;
}

int dnsmc_trace_ray(dnsmc_solver *s, int f, int g, int p, int r, int max_steps, int32_t *rec, int *n_steps,
                    uint32_t *rng4) {
    if (!s || !rec || !n_steps || max_steps < 1) return fail(DNSMC_ERR_ARG, "bad arguments");
    if (!s->solved) return fail(DNSMC_ERR_STATE, "trace needs a prior solve (sampling tables)");
    TRY(wait_done(s, 0));
    if (f < 0 || f >= s->nfields || g < 0 || g >= s->n_groups_used || r < 0) return fail(DNSMC_ERR_ARG, "trace index out of range");
    int np;
    TRY(dnsmc_packet_count(s, &np));
    if (p < 0 || p >= np) return fail(DNSMC_ERR_ARG, "packet out of range");
    if (s->mode != MODE_GREY && s->group_empty[g]) return fail(DNSMC_ERR_ARG, "band group is empty");
    TRY(set_device(s));
    int *d_rec = nullptr, *d_n = nullptr;
    unsigned int *d_rng = nullptr;
    CUDA_TRY(cudaMalloc((void **)&d_rec, (size_t)max_steps * 6 * sizeof(int)));
    cudaMalloc((void **)&d_n, sizeof(int));
    cudaMalloc((void **)&d_rng, 4 * sizeof(unsigned int));
    int rc = solve_enqueue(s, true, f, g, p, r, max_steps, d_rec, d_n, d_rng);
    if (rc == DNSMC_OK) {
        cudaError_t e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) rc = fail(DNSMC_ERR_CUDA, "trace: %s", cudaGetErrorString(e));
    }
    if (rc == DNSMC_OK) {
        cudaMemcpy(n_steps, d_n, sizeof(int), cudaMemcpyDeviceToHost);
        const int nrec = std::min(*n_steps, max_steps);
        cudaMemcpy(rec, d_rec, (size_t)nrec * 6 * sizeof(int), cudaMemcpyDeviceToHost);
        if (rng4) cudaMemcpy(rng4, d_rng, 4 * sizeof(unsigned int), cudaMemcpyDeviceToHost);
    }
    cudaFree(d_rec);
    cudaFree(d_n);
    cudaFree(d_rng);
    return rc;
}

// ---- reference drop-in ------------------------------------------------------
int dnsmc_dropin_configure(const dnsmc_config *cfg, const char *table_dir) {
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    if (g_dropin) { dnsmc_destroy(g_dropin); g_dropin = nullptr; }
    if (cfg) {
        TRY(check_config(*cfg));
        g_dropin_cfg = *cfg;
        g_dropin_cfg_set = true;
    } else {
        g_dropin_cfg_set = false;
    }
    g_dropin_tables = table_dir ? table_dir : "";
    return DNSMC_OK;
}

int dnsmc_dropin_release(void) {
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    if (g_dropin) dnsmc_destroy(g_dropin);
    g_dropin = nullptr;
    return DNSMC_OK;
}

void mc_gpu_(float *Tfort, int *ystart) {
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    if (!Tfort || !ystart) { fail(DNSMC_ERR_ARG, "null argument"); dropin_die("mc_gpu_"); }
    if (!g_dropin) {
        dnsmc_config c;
        if (g_dropin_cfg_set) {
            c = g_dropin_cfg;
        } else {
            dnsmc_set_default_config(&c);
            if (dnsmc_config_from_env(&c)) dropin_die("mc_gpu_ configuration");
        }
        if (dnsmc_create(&c, &g_dropin)) dropin_die("mc_gpu_ set-up");
        // float results with the reference's sigma normaliser, computed on
        // the device: only Q and sigma as floats cross to the host
        g_dropin->result_type = DNSMC_RESULT_F32;
        g_dropin->sig_scale = c.nvar > 1 ? (double)c.nvar / (c.nvar - 0.5) : 1.0;
        std::string dir = g_dropin_tables;
        if (dir.empty()) { const char *e = getenv("DNSMC_TABLES"); dir = e && *e ? e : "../distr/tables"; }
        int rc = DNSMC_OK;
        if (c.model == DNSMC_MODEL_CK) rc = dnsmc_load_tables_ref(g_dropin, dir.c_str(), DNSMC_MODEL_CK, 52, 119, 16);
        else if (c.model == DNSMC_MODEL_PARTICLE) rc = dnsmc_load_tables_ref(g_dropin, dir.c_str(), DNSMC_MODEL_PARTICLE, 52, 119, 1);
        else if (c.model == DNSMC_MODEL_GREY_BANDS) rc = dnsmc_use_grey_band_tables(g_dropin, 1000, 55, 15000.f, 500.f);
        else if (c.model == DNSMC_MODEL_TABLE) rc = fail(DNSMC_ERR_STATE, "the drop-in pair cannot use a raw table");
        if (rc) dropin_die("mc_gpu_ tables");
    }
    const dnsmc_config &c = g_dropin->cfg;
    const int jl = c.jmax / c.p_row;
    const int j0 = *ystart - 1;
    if (j0 < 0 || j0 + jl > c.jmax) { fail(DNSMC_ERR_ARG, "ystart %d out of range", *ystart); dropin_die("mc_gpu_"); }
    if (dnsmc_set_fields(g_dropin, 1, Tfort, nullptr, DNSMC_LAYOUT_FORTRAN)) dropin_die("mc_gpu_ fields");
    if (g_dropin->r_j0 != j0 || g_dropin->r_j1 != j0 + jl)
        if (dnsmc_set_region(g_dropin, 0, c.imax, j0, j0 + jl, 0, c.kmax)) dropin_die("mc_gpu_ region");
    if (dnsmc_solve_async(g_dropin)) dropin_die("mc_gpu_ launch");
}

void get_results_(float *resfort, float *varfort) {
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    if (!g_dropin || !g_dropin->solved) { fail(DNSMC_ERR_STATE, "get_results_ before mc_gpu_"); dropin_die("get_results_"); }
    if (wait_done(g_dropin, 0)) dropin_die("get_results_");
    const dnsmc_config &c = g_dropin->cfg;
    const int jl = c.jmax / c.p_row;
    // interior rows of imax floats into the (imax+2)(jl+2)(kmax+2) arrays
    // (code/param.h:110-111 idx_F); ghost cells stay untouched
    scatter_fortran(resfort, g_dropin->h_Qf.p, c.imax, jl, c.kmax);
    scatter_fortran(varfort, g_dropin->h_sigf.p, c.imax, jl, c.kmax);
}

}  // extern "C"
