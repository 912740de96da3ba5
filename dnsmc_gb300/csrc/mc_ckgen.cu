// mc_ckgen.cu -- correlated-k tables from line-by-line absorption spectra on
// the GPU: the reference's offline generator (distr/correlatedK.cpp:145-300,
// correlatedKT; the band means of distr/calc_prob.cpp:17-119), for every
// (temperature, H2O mole fraction, narrow band) at once.
//
// Per band of one spectrum (one CTA of 256 threads):
//   kmin, kmax over the band's points;
//   n_pwrk bins uniform in k^0.1 between kmin^0.1 and kmax^0.1; every
//   interval h of the band's points (midpoint k of points h-1 and h) lands
//   in bin 1 + floor((k^0.1 - kmin^0.1) / step) -- the reference's
//   MAX(0, (int)((kpwri - pwrk_min) / pwrk_step + 1)) -- counted in shared
//   memory;
//   the g-function g(h) = 1 - sum over bins b = h+1 .. n_pwrk-1 of the
//   spectral fraction of bin b, the fraction being count * dwv / band width
//   (the spectrum is uniform in wavenumber; the reference sums dwv / width
//   point by point, the same value up to rounding);
//   bin values k(h) = (e(h) + e(h+1)) / 2 with e(h) = (kmin^0.1 + h step)^10
//   (ten-fold products, not a power function: the host oracle gives the
//   same bits);
//   k at every quadrature point g_r by linear interpolation in g between
//   the bins that bracket it (the first h with g(h+1) >= g_r);
//   the band mean of k, sum over bins 1 .. n_pwrk-1 of k(h) x fraction(h),
//   in bin order by one thread (calc_prob.cpp's k_avg).
// Compiled with -fmad=false like the marches: the oracle (oracle/mc_oracle.cpp,
// orc_ck_from_lbl, built with -ffp-contract=off) reproduces every value up
// to the power k^0.1 of the bin boundaries.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <vector>

#include "../../include/dnsmc.h"
#include "mc_internal.h"

namespace dnsmc {

int report_error(int code, const char *msg);  // mc_host.cpp

namespace {

constexpr int kCkThreads = 256;

struct CkGenParams {
    const double *kappa;      // [nT][nX][npts]
    long long npts;
    int nT, nX, nbands, nq, n_pwrk;
    const long long *first;   // [nbands]
    const int *count;         // [nbands]
    const double *frac;       // [nbands] dwv / (wv_right - wv_left)
    const double *gq;         // [nq]
    float *kq;                // [nbands][nq][nT][nX]
    double *kavg;             // [nT][nX][nbands] or null
};

// (p0 + h * step)^10 as products
__device__ __forceinline__ double ck_edge(double p0, double step, int h) {
    const double x = (double)h * step + p0;
    const double x2 = x * x;
    const double x4 = x2 * x2;
    const double x5 = x4 * x;
    return x5 * x5;
}

__device__ __forceinline__ double ck_bin_k(double p0, double step, int h) {
    return 0.5 * (ck_edge(p0, step, h) + ck_edge(p0, step, h + 1));
}

__global__ void __launch_bounds__(kCkThreads) ck_distribution_kernel(const CkGenParams P) {
    extern __shared__ unsigned int s_cnt[];   // n_pwrk + 2 counts, then suffix sums
    __shared__ double s_red[2][kCkThreads / 32];
    __shared__ unsigned int s_part[kCkThreads];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long item = blockIdx.x;        // (t * nX + x) * nbands + band
    const int band = (int)(item % P.nbands);
    const long long tx = item / P.nbands;
    const double *kv = P.kappa + tx * P.npts + P.first[band];
    const int n = P.count[band];
    const int NB = P.n_pwrk;

    // kmin, kmax over the band's points
    double lo = INFINITY, hi = -INFINITY;
    for (int h = tid; h < n; h += kCkThreads) {
        const double v = kv[h];
        lo = fmin(lo, v);
        hi = fmax(hi, v);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if (lane == 0) { s_red[0][warp] = lo; s_red[1][warp] = hi; }
    for (int b = tid; b < NB + 2; b += kCkThreads) s_cnt[b] = 0u;
    __syncthreads();
    lo = s_red[0][0];
    hi = s_red[1][0];
    for (int w = 1; w < kCkThreads / 32; ++w) { lo = fmin(lo, s_red[0][w]); hi = fmax(hi, s_red[1][w]); }
    const int t_ = (int)(tx / P.nX), x_ = (int)(tx % P.nX);
    const long long TX = (long long)P.nT * P.nX;
    if (!(hi > lo)) {  // a flat band: k is the same at every g
        if (tid < P.nq) P.kq[((long long)band * P.nq + tid) * TX + t_ * P.nX + x_] = (float)lo;
        if (tid == 0 && P.kavg) P.kavg[tx * P.nbands + band] = lo;
        return;
    }
    const double p0 = pow(lo, 0.1), p1 = pow(hi, 0.1);
    const double step = (p1 - p0) / (double)(NB - 1);
    // bins of the intervals between neighbouring points
    for (int h = 1 + tid; h < n; h += kCkThreads) {
        const double ki = (kv[h] + kv[h - 1]) / 2.0;
        int b = (int)((pow(ki, 0.1) - p0) / step + 1.0);
        b = min(max(b, 0), NB);
        atomicAdd(&s_cnt[b], 1u);
    }
    __syncthreads();
    // suffix sums over bins 1 .. NB-1 (the bins the g-function uses):
    // s_cnt[h] <- sum_{b = h .. NB-1} count[b] for h = 1 .. NB, 0 at NB
    {
        const int per = (NB + kCkThreads - 1) / kCkThreads;
        const int b0 = 1 + tid * per, b1 = min(NB, b0 + per);  // this thread's bins [b0, b1)
        unsigned int acc = 0;
        for (int b = b0; b < b1; ++b) acc += s_cnt[b];
        s_part[tid] = acc;
        __syncthreads();
        unsigned int above = 0;  // bins after this thread's chunk
        for (int q = tid + 1; q < kCkThreads; ++q) above += s_part[q];
        __syncthreads();
        unsigned int run = above;
        for (int b = b1 - 1; b >= b0; --b) {
            run += s_cnt[b];
            s_cnt[b] = run;
        }
        if (tid == 0) s_cnt[NB] = 0u;
        __syncthreads();
    }
    const double frac = P.frac[band];
    // g(h) = 1 - (suffix count from h + 1) x frac, h = 0 .. NB-1
    auto g_at = [&](int h) -> double { return 1.0 - (double)s_cnt[h + 1] * frac; };
    if (tid < P.nq) {
        const double g = P.gq[tid];
        // first t in [0, NB-2] with g(t+1) >= g (g(NB-1) = 1 >= g)
        int a = 0, z = NB - 2;
        while (a < z) {
            const int m = (a + z) >> 1;
            if (g_at(m + 1) >= g) z = m; else a = m + 1;
        }
        const int t = a;
        const double g0 = g_at(t), g1 = g_at(t + 1);
        const double k0 = ck_bin_k(p0, step, t), k1 = ck_bin_k(p0, step, t + 1);
        const double kq = (g1 == g0) ? k1 : k0 + (k1 - k0) * (g - g0) / (g1 - g0);
        P.kq[((long long)band * P.nq + tid) * TX + t_ * P.nX + x_] = (float)kq;
    }
    if (tid == 0 && P.kavg) {
        double s = 0.0;
        for (int h = 1; h < NB; ++h) {
            const unsigned int c = s_cnt[h] - s_cnt[h + 1];
            if (c) s += ck_bin_k(p0, step, h) * ((double)c * frac);
        }
        P.kavg[tx * P.nbands + band] = s;
    }
}

template <class T>
struct Dev {
    T *p = nullptr;
    ~Dev() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t n) { return cudaMalloc((void **)&p, (n ? n : 1) * sizeof(T)); }
};

}  // namespace
}  // namespace dnsmc

using namespace dnsmc;

extern "C" int dnsmc_ck_from_lbl(const dnsmc_lbl_desc *d, float *kq, double *kavg) {
    if (!d || !kq || !d->kappa || !d->first || !d->count || !d->wv_left || !d->wv_right || !d->gq)
        return report_error(DNSMC_ERR_ARG, "null argument");
    if (d->nT < 1 || d->nX < 1 || d->npts < 2 || d->nbands < 1 || d->nq < 1 || d->n_pwrk < 2)
        return report_error(DNSMC_ERR_ARG, "sizes must be >= 1 (npts, n_pwrk >= 2)");
    if (!(d->dwv > 0)) return report_error(DNSMC_ERR_ARG, "dwv must be > 0");
    // the bin counts live in shared memory
    if (d->n_pwrk > 50000) return report_error(DNSMC_ERR_ARG, "n_pwrk must be <= 50000");
    std::vector<double> frac((size_t)d->nbands);
    for (int b = 0; b < d->nbands; ++b) {
        if (d->count[b] < 2 || d->first[b] < 0 || d->first[b] + d->count[b] > d->npts)
            return report_error(DNSMC_ERR_ARG, "every band needs >= 2 points inside the spectrum");
        const double w = d->wv_right[b] - d->wv_left[b];
        if (!(w > 0)) return report_error(DNSMC_ERR_ARG, "band edges must satisfy wv_left < wv_right");
        frac[(size_t)b] = d->dwv / w;
    }
    for (int r = 0; r < d->nq; ++r)
        if (!(d->gq[r] > 0) || !(d->gq[r] < 1) || (r && !(d->gq[r] > d->gq[r - 1])))
            return report_error(DNSMC_ERR_ARG, "quadrature points must ascend inside (0, 1)");
    const long long nk = (long long)d->nT * d->nX * d->npts;
    for (long long i = 0; i < nk; ++i)
        if (!(d->kappa[i] >= 0) || !std::isfinite(d->kappa[i]))
            return report_error(DNSMC_ERR_TABLE, "absorption spectra must be finite and >= 0");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return report_error(DNSMC_ERR_NODEVICE, "no CUDA device");
    Dev<double> dk, dfrac, dgq, dkavg;
    Dev<long long> dfirst;
    Dev<int> dcount;
    Dev<float> dkq;
    const long long items = (long long)d->nT * d->nX * d->nbands;
    cudaError_t e = dk.alloc((size_t)nk);
    if (e == cudaSuccess) e = dfrac.alloc((size_t)d->nbands);
    if (e == cudaSuccess) e = dgq.alloc((size_t)d->nq);
    if (e == cudaSuccess) e = dfirst.alloc((size_t)d->nbands);
    if (e == cudaSuccess) e = dcount.alloc((size_t)d->nbands);
    if (e == cudaSuccess) e = dkq.alloc((size_t)items * d->nq);
    if (e == cudaSuccess && kavg) e = dkavg.alloc((size_t)items);
    if (e != cudaSuccess) return report_error(DNSMC_ERR_NOMEM, cudaGetErrorString(e));
    e = cudaMemcpy(dk.p, d->kappa, (size_t)nk * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dfrac.p, frac.data(), frac.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dgq.p, d->gq, (size_t)d->nq * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dfirst.p, d->first, (size_t)d->nbands * sizeof(long long), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dcount.p, d->count, (size_t)d->nbands * sizeof(int), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return report_error(DNSMC_ERR_CUDA, cudaGetErrorString(e));
    CkGenParams P{};
    P.kappa = dk.p; P.npts = d->npts; P.nT = d->nT; P.nX = d->nX; P.nbands = d->nbands; P.nq = d->nq;
    P.n_pwrk = d->n_pwrk; P.first = dfirst.p; P.count = dcount.p; P.frac = dfrac.p; P.gq = dgq.p;
    P.kq = dkq.p; P.kavg = kavg ? dkavg.p : nullptr;
    const size_t smem = (size_t)(d->n_pwrk + 2) * sizeof(unsigned int);
    if (smem > 48 * 1024) {
        e = cudaFuncSetAttribute(ck_distribution_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return report_error(DNSMC_ERR_ARG, "n_pwrk too large for shared memory");
    }
    if (items > 0x7fffffffLL) return report_error(DNSMC_ERR_ARG, "too many (T, x, band) items");
    dnsmc::note_launch();
    ck_distribution_kernel<<<(unsigned)items, kCkThreads, smem>>>(P);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(kq, dkq.p, (size_t)items * d->nq * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && kavg) e = cudaMemcpy(kavg, dkavg.p, (size_t)items * sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return report_error(DNSMC_ERR_CUDA, cudaGetErrorString(e));
    return DNSMC_OK;
}
