// mc_oracle.cpp -- TEST INFRASTRUCTURE ONLY.  CPU restatement of the
// reference reverse Monte Carlo of simone-silvestri/dnsMC, used by tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker.
// Nothing in the product (dnsmc_gb300/) links or calls it.
//
// Three parts:
//  (1) orc_ref_mc: the reference estimator in the reference's own structure
//      -- one thread per cell, nVar batches of photmax rays
//      (code/mc_gpu.cu:44-226), emission direction (:813-820), band and
//      g-point bisection on the CDF at the table temperature nearest Tmax
//      (:830-896), the OERM weights (:59-63, :162-169), the position-update
//      voxel march with periodic and black-wall boundaries (:228-438), the
//      multigrid switch (:193-207) on spline-coarsened temperature
//      (code/spline.cpp:35-170), linear-filter table lookups with clamp
//      addressing (code/memory_copy.cu:131-289) optionally with the 8-bit
//      fixed-point filter weights of the texture unit.  Templated on the
//      arithmetic type: FP32 reproduces the reference build (the timed CPU
//      baseline), FP64 is the oracle.  curand is replaced by Philox4x32-10
//      streams keyed per (cell, batch, ray): the reference's stream is not
//      reproducible (colliding seeds, code/mc_gpu.cu:99), so comparisons with
//      it are statistical.
//  (2) orc_packet_mc / orc_packet_trace: an independent restatement of the
//      GB300 packet scheme (32, 64 or 128 cells of one wall-normal plane
//      share each ray's direction and spectral sample) that reproduces the
//      device march bit for bit in FP32 (same Philox counters, same alias
//      draw, same fmaf-based polynomial exp/sin/cos, the same float-pair
//      per-ray sums), or runs it in FP64; orc_cv_table builds the control
//      variate's surrogate table by the device's FP32 sweeps, orc_cv_mean
//      the FP64 solution's own exact means.
//  (3) helpers: Philox4x32-10, the reference grids, the spline; the
//      k-distribution of line-by-line spectra (orc_ck_from_lbl).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <type_traits>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): 10 rounds of the 4x32
// Philox S-box with multipliers D2511F53, CD9E8D57 and Weyl key increments
// 9E3779B9, BB67AE85.
// ---------------------------------------------------------------------------
static inline void philox(const uint32_t in[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
    uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        const uint32_t n1 = (uint32_t)p1;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        const uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { philox(ctr, key[0], key[1], out); }

// ---------------------------------------------------------------------------
// Reference grids (code/definitions.h:68-136): stretched wall-normal faces
// for im cells taken from the im0 fine grid, uniform periodic faces.
// ---------------------------------------------------------------------------
void orc_ref_faces(int im, int im0, float L, int stretched, float *xu) {
    if (!stretched) {
        for (int i = 0; i <= im; ++i) xu[i] = (float)i * (L / (float)im);
        xu[im] = L;
        return;
    }
    std::vector<float> xu0(im0 + 1, 0.0f);
    for (int i = 1; i < im0 / 2 + 1; ++i) {
        const float r = (1.f * i) / im0;
        const float dx = (float)(0.5 - 1.45 * (r - 0.5) * (r - 0.5));
        xu0[i] = xu0[i - 1] + dx;
    }
    const float xnorm = xu0[im0 / 2];
    for (int i = 1; i < im0 / 2 + 1; ++i) xu0[i] = (float)(L / 2. * xu0[i] / xnorm);
    for (int i = im0; i > im0 / 2; --i) xu0[i] = L - xu0[im0 - i];
    xu[0] = 0;
    for (int i = 1; i < im + 1; ++i) xu[i] = xu0[i * im0 / im];
}

}  // extern "C"

namespace {

struct Grid {  // one level, reference Gridn + Var_CPU (1-based cells, ghosts at 0, n+1)
    int im, jm, km, sm;
    std::vector<float> x, xu, y, yu, z, zu, T;
};

void mk_grid(Grid &g, int im, int jm, int km, int im0, int sm, float Lx, float Ly, float Lz, int stretched) {
    g.im = im; g.jm = jm; g.km = km; g.sm = sm;
    g.x.assign(im + 2, 0.f); g.xu.assign(im + 1, 0.f);
    g.y.assign(jm + 2, 0.f); g.yu.assign(jm + 1, 0.f);
    g.z.assign(km + 2, 0.f); g.zu.assign(km + 1, 0.f);
    const float dy = Ly / jm, dz = Lz / km;
    for (int i = 0; i < jm + 1; ++i) g.yu[i] = i * dy;
    for (int i = 0; i < km + 1; ++i) g.zu[i] = i * dz;
    g.y[0] = -dy / 2; g.z[0] = -dz / 2;
    for (int i = 1; i < jm + 1; ++i) g.y[i] = (g.yu[i - 1] + g.yu[i]) / 2;
    for (int i = 1; i < km + 1; ++i) g.z[i] = (g.zu[i - 1] + g.zu[i]) / 2;
    g.y[jm + 1] = g.y[jm] + dy; g.z[km + 1] = g.z[km] + dz;
    orc_ref_faces(im, im0, Lx, stretched, g.xu.data());
    for (int i = 1; i < im + 1; ++i) g.x[i] = (float)(0.5 * (g.xu[i] + g.xu[i - 1]));
    g.x[0] = -g.x[1];
    g.x[im + 1] = g.xu[im] + (g.xu[im] - g.x[im]);
    g.T.assign((size_t)(im + 2) * (jm + 2) * (km + 2), 0.f);
}

inline size_t idxT(int i, int j, int k, int im, int jm) { return i + (size_t)(im + 2) * (j + (size_t)k * (jm + 2)); }

// Natural cubic spline on 1-based arrays (Numerical Recipes, as code/spline.cpp:119-170).
void spline(const float *x, const float *y, int n, float *y2) {
    std::vector<float> u(n + 1);
    y2[1] = u[1] = 0.0f;
    for (int i = 2; i <= n - 1; ++i) {
        const float sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
        const float p = sig * y2[i - 1] + 2.0f;
        y2[i] = (sig - 1.0f) / p;
        float ui = (y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1]);
        u[i] = (float)((6.0 * ui / (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / p);
    }
    y2[n] = 0.0f;
    for (int k = n - 1; k >= 1; --k) y2[k] = y2[k] * y2[k + 1] + u[k];
}

float splint(const float *xa, const float *ya, const float *y2a, int n, float x) {
    int klo = 1, khi = n;
    while (khi - klo > 1) {
        const int k = (khi + klo) >> 1;
        if (xa[k] > x) khi = k; else klo = k;
    }
    const float h = xa[khi] - xa[klo];
    const float a = (xa[khi] - x) / h, b = (x - xa[klo]) / h;
    return (float)(a * ya[klo] + b * ya[khi] + ((a * a * a - a) * y2a[klo] + (b * b * b - b) * y2a[khi]) * (h * h) / 6.0);
}

// Separable spline coarsening of the fine temperature (code/spline.cpp:35-116).
void interp3d(std::vector<Grid> &g) {
    const Grid &f = g[0];
    const int I = f.im, J = f.jm, K = f.km;
    const int ng = (int)g.size();
    std::vector<std::vector<float>> tx(ng), txy(ng);
    for (int l = 1; l < ng; ++l) {
        tx[l].assign((size_t)(g[l].im + 2) * (J + 2) * (K + 2), 0.f);
        txy[l].assign((size_t)(g[l].im + 2) * (g[l].jm + 2) * (K + 2), 0.f);
    }
    std::vector<float> a(std::max({I, J, K}) + 2), a2(std::max({I, J, K}) + 2);
    for (int j = 1; j <= J; ++j)
        for (int k = 1; k <= K; ++k) {
            for (int i = 1; i <= I; ++i) a[i] = f.T[idxT(i, j, k, I, J)];
            spline(f.x.data(), a.data(), I, a2.data());
            for (int l = 1; l < ng; ++l)
                for (int i = 1; i <= g[l].im; ++i)
                    tx[l][idxT(i, j, k, g[l].im, J)] = splint(f.x.data(), a.data(), a2.data(), I, g[l].x[i]);
        }
    for (int l = 1; l < ng; ++l)
        for (int i = 1; i <= g[l].im; ++i)
            for (int k = 1; k <= K; ++k) {
                for (int j = 1; j <= J; ++j) a[j] = tx[l][idxT(i, j, k, g[l].im, J)];
                spline(f.y.data(), a.data(), J, a2.data());
                for (int j = 1; j <= g[l].jm; ++j)
                    txy[l][idxT(i, j, k, g[l].im, g[l].jm)] = splint(f.y.data(), a.data(), a2.data(), J, g[l].y[j]);
            }
    for (int l = 1; l < ng; ++l)
        for (int i = 1; i <= g[l].im; ++i)
            for (int j = 1; j <= g[l].jm; ++j) {
                for (int k = 1; k <= K; ++k) a[k] = txy[l][idxT(i, j, k, g[l].im, g[l].jm)];
                spline(f.z.data(), a.data(), K, a2.data());
                for (int k = 1; k <= g[l].km; ++k)
                    g[l].T[idxT(i, j, k, g[l].im, g[l].jm)] = splint(f.z.data(), a.data(), a2.data(), K, g[l].z[k]);
            }
}

float I_blackC(float T, float nu) {
    if (!(T > 0)) return 0.0f;
    const float C1 = 3.741771790075259e-16f, C2 = 0.014387741858429f;
    const float n = nu * 100.0f;
    return (float)(1.0 / 3.14159265358979323846 * (double)C1 * (double)(n * n * n) /
                   (double)(expf(C2 * nu * 100.0f / T) - 1.0f));
}

}  // namespace

extern "C" {

// ===========================================================================
// (1) reference-structured estimator
// ===========================================================================
typedef struct {
    int imax, jmax, kmax;
    float Lx, Ly, Lz;
    int stretched;
    int grid_num;
    int maxs[6];
    float T_west, T_east;
    float toll;
    int nvar, photmax;
    int hwfilter;
    int use_double;
    uint64_t seed;
    int model;          // 0 ck, 1 grey bands (built here), 2 particle
    float kappa;        // grey-band absorption coefficient
    int nT, nB, nQ;
    const float *Tnb;   // [nT]
    const float *kq;    // [nB][nT][nQ]
    const float *wvc;   // [nB]
    const float *prob;  // [nT][nB]
    const float *probg; // [nT][nB][nQ] or NULL
    const float *kP;    // [nT]
} OrcRefConfig;

}  // extern "C"

namespace {

struct RefTables {
    int nT, nB, nQ;
    std::vector<float> Tnb, kq, wvc, prob, probg, kP, Ib, ibw_w, ibw_e;
    float Tmax, kappamax;
    int tm;
};

// Linear-filter fetch along one axis of a clamp-addressed texture at
// coordinate pos+0.5 (texel centres at integers), as the texture unit does;
// hw: quantise the fraction to 1/256 (8-bit fixed point weights).
template <class R>
inline R tex_lerp(const float *row, int stride, int n, R pos, int hw) {
    R xb = pos;  // = (pos + 0.5) - 0.5
    R fl = std::floor(xb);
    int i0 = (int)fl;
    R a = xb - fl;
    if (hw) a = std::round(a * (R)256) / (R)256;
    const int c0 = std::min(std::max(i0, 0), n - 1), c1 = std::min(std::max(i0 + 1, 0), n - 1);
    return ((R)1 - a) * (R)row[(size_t)c0 * stride] + a * (R)row[(size_t)c1 * stride];
}

template <class R>
struct RefMC {
    const OrcRefConfig &c;
    const RefTables &t;
    const std::vector<Grid> &g;
    RefMC(const OrcRefConfig &c_, const RefTables &t_, const std::vector<Grid> &g_) : c(c_), t(t_), g(g_) {}

    R kfetch(int nb, R pos, int gq) const {  // tex3D(tex, nb+.5, pos+.5, g+.5), extent (nB, nT, nQ)
        const int gg = std::min(std::max(gq, 0), t.nQ - 1);
        // kq layout [nB][nT][nQ]: along T the stride is nQ
        return tex_lerp<R>(t.kq.data() + (size_t)nb * t.nT * t.nQ + gg, t.nQ, t.nT, pos, c.hwfilter);
    }
    R ibfetch(int nb, R pos) const {  // tex2D(tex_Ib, nb+.5, pos+.5), Ib[nT][nB]
        return tex_lerp<R>(t.Ib.data() + nb, t.nB, t.nT, pos, c.hwfilter);
    }

    // find_band (code/mc_gpu.cu:830-896)
    void find_band(R u1, R u2, int *nb, int *gq) const {
        const int tm = t.tm;
        const R T0 = t.Tnb[tm], T1 = t.Tnb[tm + 1];
        const int ts = ((R)t.Tmax - T0) < (T1 - (R)t.Tmax) ? tm : tm + 1;
        const float *pd = t.prob.data() + (size_t)ts * t.nB;
        int lo = 0, w = t.nB;
        while (w > lo + 1) {
            const int d = (lo + w) / 2;
            if (u1 < (R)pd[d]) w = d; else lo = d;
        }
        lo = lo + 1;
        if (u1 < (R)pd[0]) lo = 0;
        if (u1 == (R)1) lo = t.nB - 1;
        *nb = lo;
        if (c.model == 1) { *gq = 0; return; }
        int gg = 0;
        w = t.nQ;
        const float *pg = t.probg.empty() ? nullptr : t.probg.data() + ((size_t)ts * t.nB + lo) * t.nQ;
        while (w > gg + 1) {
            const int d = (gg + w) / 2;
            const R pr = pg ? (R)pg[d] : (R)0;
            if (u2 < pr) w = d; else gg = d;
        }
        gg = gg + 1;
        const R p0 = pg ? (R)pg[0] : (R)0;
        if (u2 < p0) gg = 0;
        if (u2 == (R)1) gg = t.nQ - 1;
        *gq = gg;  // may equal nQ (reference behaviour for nQ == 1); fetches clamp
    }

    void cell(int ci, int cj, int ck, uint64_t cell_id, double *sol, double *var, double *se, double *nsteps) const {
        const R pi = (R)3.14159265358979323846;
        const R stefan = (R)5.670373e-08;
        const Grid &g0 = g[0];
        const R dT = (R)t.Tnb[1] - (R)t.Tnb[0];
        const R Tnb0 = (R)t.Tnb[0];
        const R Tn0 = dT, Tn1 = Tnb0 / dT;  // code/mc_gpu.cu:59
        const R Ibmax = (R)4 * (R)t.kappamax * (R)t.Tmax * (R)t.Tmax * (R)t.Tmax * (R)t.Tmax * stefan / (R)c.photmax;
        const R Ti = (R)g0.T[idxT(ci, cj, ck, g0.im, g0.jm)];
        std::vector<R> Dv(c.nvar, (R)0);
        double sum = 0, sum2 = 0, steps = 0;
        const uint32_t k0 = (uint32_t)c.seed, k1 = (uint32_t)(c.seed >> 32);
        for (int v = 0; v < c.nvar; ++v) {
            R De = 0;
            for (int h = 0; h < c.photmax; ++h) {
                const uint32_t ctr[4] = {(uint32_t)h, (uint32_t)v, (uint32_t)cell_id, (uint32_t)(cell_id >> 32) ^ 0x5EF0u};
                uint32_t rn[4];
                philox(ctr, k0, k1, rn);
                // curand_uniform is in (0, 1]
                auto U = [](uint32_t x) { return (R)((x >> 8) + 1) * (R)5.9604644775390625e-8; };
                R xp = g0.x[ci], yp = g0.y[cj], zp = g0.z[ck];
                int ic = ci, jc = cj, kc = ck;
                const R phi = U(rn[0]) * (R)2 * pi;
                const R theta = std::acos((R)1 - (R)2 * U(rn[1]));
                R sx = std::cos(theta), sy = std::sin(theta) * std::cos(phi), sz = std::sin(theta) * std::sin(phi);
                if (sx == 0) sx = (R)1e-10;
                if (sy == 0) sy = (R)1e-10;
                if (sz == 0) sz = (R)1e-10;
                const int fl[3] = {sx < 0, sy < 0, sz < 0};
                int nb, gq;
                find_band(U(rn[2]), U(rn[3]), &nb, &gq);
                R tra = 1;
                R pos = (Ti - Tnb0) / dT;
                const R a2 = kfetch(nb, pos, gq);
                const R invTi4 = (R)1 / ibfetch(nb, pos);
                pos = ((R)t.Tmax - Tnb0) / dT;
                const R a1 = kfetch(nb, pos, gq);
                const R ratioI = ((R)1 / invTi4) / ibfetch(nb, pos) * a2 / a1;
                // start-cell fix-ups (code/mc_gpu.cu:174-186)
                if (fl[0] && xp == (R)g0.xu[ic - 1]) ic--;
                if (fl[1] && yp == (R)g0.yu[jc - 1]) jc--;
                if (fl[2] && zp == (R)g0.zu[kc - 1]) kc--;
                if (!fl[0] && xp == (R)g0.xu[ic]) ic++;
                if (!fl[1] && yp == (R)g0.yu[jc]) jc++;
                if (!fl[2] && zp == (R)g0.zu[kc]) kc++;
                const R before = De;
                for (int grd = 0; grd < (int)g.size(); ++grd) {
                    const Grid &G = g[grd];
                    int counter = 0;
                    while (tra > (R)c.toll && counter < G.sm) {
                        const R dsx = ((R)G.xu[ic - fl[0]] - xp) / sx;
                        const R dsy = ((R)G.yu[jc - fl[1]] - yp) / sy;
                        const R dsz = ((R)G.zu[kc - fl[2]] - zp) / sz;
                        const R tf = (R)G.T[idxT(ic, jc, kc, G.im, G.jm)];
                        const R p2 = tf / Tn0 - Tn1;
                        const R absco = kfetch(nb, p2, gq);
                        const R bp = ibfetch(nb, p2);
                        R ds = dsx;
                        if (ds > dsy) ds = dsy;
                        if (ds > dsz) ds = dsz;
                        if (ds == dsx) xp = G.xu[ic - fl[0]]; else xp = xp + ds * sx;
                        if (ds == dsy) yp = G.yu[jc - fl[1]]; else yp = yp + ds * sy;
                        if (ds == dsz) zp = G.zu[kc - fl[2]]; else zp = zp + ds * sz;
                        const R alpha = (R)1 - std::exp(-ds * absco);
                        De -= Ibmax * tra * alpha * ratioI * (invTi4 * bp - (R)1);
                        tra = tra * ((R)1 - alpha);
                        if (tra < (R)c.toll) {
                            De -= Ibmax * tra * ratioI * (invTi4 * bp - (R)1);
                            tra = 0;
                        }
                        if (dsx < dsy) {
                            if (dsx < dsz) {
                                if (fl[0]) {
                                    ic--;
                                    if (ic == 0) { De -= Ibmax * tra * (invTi4 * (R)t.ibw_w[nb] - (R)1) * ratioI; tra = 0; }
                                } else {
                                    ic++;
                                    if (ic == G.im + 1) { De -= Ibmax * tra * (invTi4 * (R)t.ibw_e[nb] - (R)1) * ratioI; tra = 0; }
                                }
                            } else {
                                if (fl[2]) { kc--; if (kc == 0) { kc = G.km; zp = c.Lz; } }
                                else { kc++; if (kc == G.km + 1) { kc = 1; zp = 0; } }
                            }
                        } else {
                            if (dsy < dsz) {
                                if (fl[1]) { jc--; if (jc == 0) { jc = G.jm; yp = c.Ly; } }
                                else { jc++; if (jc == G.jm + 1) { jc = 1; yp = 0; } }
                            } else {
                                if (fl[2]) { kc--; if (kc == 0) { kc = G.km; zp = c.Lz; } }
                                else { kc++; if (kc == G.km + 1) { kc = 1; zp = 0; } }
                            }
                        }
                        ++counter;
                        steps += 1;
                    }
                    if (grd < (int)g.size() - 1) {
                        const int ri = G.im / g[grd + 1].im, rj = G.jm / g[grd + 1].jm, rk = G.km / g[grd + 1].km;
                        ic = (ic + ri - 1) / ri; jc = (jc + rj - 1) / rj; kc = (kc + rk - 1) / rk;
                    }
                }
                const double xr = (double)(De - before) * c.photmax;
                sum += xr;
                sum2 += xr * xr;
            }
            Dv[v] = De;
        }
        R sol_ = 0;
        for (int v = 0; v < c.nvar; ++v) sol_ += Dv[v];
        sol_ /= (R)c.nvar;
        double var_ = 0;
        for (int v = 0; v < c.nvar; ++v)
            var_ += 1. / (c.nvar - 0.5) * 1. / (c.nvar - 1) * (double)(Dv[v] - sol_) * (double)(Dv[v] - sol_);
        const double n = (double)c.nvar * c.photmax;
        const double m = sum / n;
        *sol = (double)sol_;
        *var = c.nvar > 1 ? var_ : 0.0;
        *se = n > 1 ? std::sqrt(std::max(0.0, sum2 / n - m * m) / (n - 1)) : 0.0;
        *nsteps = steps;
    }
};

int build_ref_tables(const OrcRefConfig &c, const std::vector<Grid> &g, RefTables &t) {
    // Tmax over interior cells and walls (code/mc_gpu.cu:470-486)
    const Grid &f = g[0];
    float Tmax = 0;
    for (int k = 1; k <= f.km; ++k)
        for (int j = 1; j <= f.jm; ++j)
            for (int i = 1; i <= f.im; ++i) Tmax = std::max(Tmax, f.T[idxT(i, j, k, f.im, f.jm)]);
    Tmax = std::max(Tmax, std::max(c.T_west, c.T_east));
    t.Tmax = Tmax;
    if (c.model == 1) {  // code/grey_tables.cpp:19-109
        const int nB = 1000, nT = 55;
        const float wvmax = 15000.f, Tmins = 500.f;
        t.nB = nB; t.nT = nT; t.nQ = 1;
        t.Tnb.resize(nT);
        for (int i = 0; i < nT; ++i) t.Tnb[i] = Tmins * 0.9f + (Tmax * 1.1f - Tmins * 0.9f) * ((float)i) / ((float)nT);
        std::vector<float> wvl(nB), wvr(nB);
        wvl[0] = 0;
        for (int i = 1; i < nB; ++i) wvl[i] = wvl[i - 1] + wvmax / nB;
        wvr[0] = wvmax / nB;
        for (int i = 1; i < nB; ++i) wvr[i] = wvr[i - 1] + wvmax / nB;
        t.wvc.resize(nB);
        for (int i = 0; i < nB; ++i) t.wvc[i] = (float)((wvl[i] + wvr[i]) / 2.);
        t.kq.assign((size_t)nB * nT, c.kappa);
        t.kP.assign(nT, c.kappa);
        t.prob.assign((size_t)nT * nB, 0.f);
        for (int i = 0; i < nT; ++i) {
            float acc = I_blackC(t.Tnb[i], t.wvc[0]) * (wvr[0] - wvl[0]) * 100;
            t.prob[(size_t)i * nB] = acc;
            for (int b = 1; b < nB; ++b) {
                acc = acc + I_blackC(t.Tnb[i], t.wvc[b]) * (wvr[b] - wvl[b]) * 100;
                t.prob[(size_t)i * nB + b] = acc;
            }
            const float last = t.prob[(size_t)i * nB + nB - 1];
            for (int b = 0; b < nB; ++b) t.prob[(size_t)i * nB + b] /= last;
        }
        t.kappamax = c.kappa;
    } else {
        t.nB = c.nB; t.nT = c.nT; t.nQ = c.nQ;
        t.Tnb.assign(c.Tnb, c.Tnb + c.nT);
        t.kq.assign(c.kq, c.kq + (size_t)c.nB * c.nT * c.nQ);
        t.wvc.assign(c.wvc, c.wvc + c.nB);
        t.prob.assign(c.prob, c.prob + (size_t)c.nT * c.nB);
        if (c.probg) t.probg.assign(c.probg, c.probg + (size_t)c.nT * c.nB * c.nQ);
        t.kP.assign(c.kP, c.kP + c.nT);
        int tk = (int)((Tmax - t.Tnb[0]) / (t.Tnb[1] - t.Tnb[0]));
        tk = std::max(0, std::min(tk, t.nT - 2));
        t.kappamax = (t.kP[tk + 1] - t.kP[tk]) / (t.Tnb[tk + 1] - t.Tnb[tk]) * (Tmax - t.Tnb[tk]) + t.kP[tk];
    }
    t.tm = (int)((Tmax - t.Tnb[0]) / (t.Tnb[1] - t.Tnb[0]));
    t.tm = std::max(0, std::min(t.tm, t.nT - 2));
    t.Ib.assign((size_t)t.nT * t.nB, 0.f);
    for (int i = 0; i < t.nT; ++i)
        for (int b = 0; b < t.nB; ++b) t.Ib[(size_t)i * t.nB + b] = I_blackC(t.Tnb[i], t.wvc[b]);
    t.ibw_w.resize(t.nB); t.ibw_e.resize(t.nB);
    for (int b = 0; b < t.nB; ++b) { t.ibw_w[b] = I_blackC(c.T_west, t.wvc[b]); t.ibw_e[b] = I_blackC(c.T_east, t.wvc[b]); }
    return 0;
}

}  // namespace

extern "C" {

// Tfort: (imax+2)(jmax+2)(kmax+2), i fastest, with ghosts.  cells: 3*ncells
// 1-based (i, j, k).  Outputs per cell: reference batch mean, reference
// variance (normaliser 1/((nVar-0.5)(nVar-1))), per-ray standard error, steps.
int orc_ref_mc(const OrcRefConfig *c, const float *Tfort, int ncells, const int *cells, int nthreads,
               double *sol, double *var, double *se, double *steps) {
    if (!c || !Tfort || !cells || c->grid_num < 1 || c->grid_num > 6) return 1;
    std::vector<Grid> g(c->grid_num);
    for (int l = 0; l < c->grid_num; ++l) {
        const int sh = 1 << l;
        mk_grid(g[l], c->imax / sh, c->jmax / sh, c->kmax / sh, c->imax, c->maxs[l], c->Lx, c->Ly, c->Lz, c->stretched);
    }
    memcpy(g[0].T.data(), Tfort, g[0].T.size() * sizeof(float));
    if (c->grid_num > 1) interp3d(g);
    RefTables t;
    build_ref_tables(*c, g, t);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 1)
    for (int n = 0; n < ncells; ++n) {
        const int i = cells[3 * n], j = cells[3 * n + 1], k = cells[3 * n + 2];
        const uint64_t id = (uint64_t)i + (uint64_t)(c->imax + 2) * ((uint64_t)j + (uint64_t)(c->jmax + 2) * k);
        if (c->use_double) RefMC<double>(*c, t, g).cell(i, j, k, id, sol + n, var + n, se + n, steps + n);
        else RefMC<float>(*c, t, g).cell(i, j, k, id, sol + n, var + n, se + n, steps + n);
    }
    return 0;
}

// Spline-coarsened temperature of level `level` (for tests of interp3D).
int orc_coarsen(int imax, int jmax, int kmax, float Lx, float Ly, float Lz, int stretched, int grid_num,
                const float *Tfort, int level, float *Tout) {
    if (level < 0 || level >= grid_num) return 1;
    std::vector<Grid> g(grid_num);
    for (int l = 0; l < grid_num; ++l) {
        const int sh = 1 << l;
        mk_grid(g[l], imax / sh, jmax / sh, kmax / sh, imax, 1, Lx, Ly, Lz, stretched);
    }
    memcpy(g[0].T.data(), Tfort, g[0].T.size() * sizeof(float));
    interp3d(g);
    memcpy(Tout, g[level].T.data(), g[level].T.size() * sizeof(float));
    return 0;
}

// ===========================================================================
// (2) packet scheme replay
// ===========================================================================
typedef struct {
    int nw, na, nb;
    float da, db;
    const float *fw;          // nw+1
    int ew0, ew1, ea0, ea1, eb0, eb1;
    int tile_a;
    int mode;                 // 0 grey, 1 table(T), 2 table(T, x)
    int nfields;
    const float *fieldT;      // [f][k][j][i] dense, i fastest
    const float *fieldX;      // same, or NULL
    int nbands, nq, nT, nX;
    float T0, dT, X0, dX;
    const float *ktab;        // [band][g][t][x]
    const float *ibtab;       // [band][t]
    const float *ibw;         // [2][band]
    int n_groups;
    const int *group_start;   // n_groups+1
    const float *prob;        // alias thresholds
    const int *alias;
    const int *band;
    const int *gq;
    const float *W;
    float kappa;
    float T_west, T_east;
    int rays;
    const int *rays_per_packet;  // [G * rays_gstride + packet]
    int rays_gstride;            // 0: per packet; npackets: per (group, packet)
    uint64_t seed;
    float toll;
    int max_steps;
    int use_double;
    int sampler;              // 0: Philox iid, 1: digitally shifted Sobol' net (RQMC)
    int nbatch;               // RQMC replicates per (packet, group)
    int n_tbins;              // >0: sampling tables per temperature bin
    int cv;                   // 1: tally X - beta*Y, Y = the same ray through the layer-mean profile
    const float *sur_k;       // [field][sample][nw] layer-mean absorption coefficient
    const float *sur_I;       // [field][sample][nw] layer-mean band intensity
    const float *beta;        // [field][group][k][j][i][2] (beta_a, beta_b) dense, or NULL (1, -1)
    double *moments;          // optional [f][G][tc][9]: sums X, Ya, Yb, X^2, Ya^2, Yb^2, X Ya, X Yb, Ya Yb
    // general medium (particles with scattering, grey walls)
    int gen;
    const float *fieldV;      // dense like fieldT: particle volume fraction, or NULL
    const float *part;        // [band][2]: absorption, scattering per unit volume fraction
    float fv_max, hg_g;
    float eps[2];
    // multigrid: levels 1..mg_levels-1, 2x coarser per axis each
    int mg_levels, mg_steps;
    const float *mgT;         // coarse T, level l at mg_off[l]: [f][i][k][j]
    const float *mgfw;        // coarse wall-normal faces, level l at mg_fwoff[l]
    long long mg_off[6];
    int mg_fwoff[6];
    float mg_da[6], mg_db[6];
    float Ly, Lz;
    int cpl;                  // cells per lane (1, 2 or 4): a packet is 32 * cpl cells (tile_a x tile_b)
    int pw_step;              // > 1 (orc_packet_mc, orc_cv_mean): only every pw_step-th wall-normal layer
                              // of the region, from ew0, with the rays of an unstrided run
    const float *sur_tab;     // cv = 1: the surrogate table of orc_cv_table [field][sample][nw][2][kSurBinsO][4],
                              // read like the march does; NULL: the walk itself at the ray's cosine
} OrcPacketConfig;

}  // extern "C"

namespace {

// Own polynomial exp/sin/cos of the packet specification (FP32, fmaf only).
inline float p_expm1(float x) {
    x = std::fmax(x, -87.0f);
    // n rounded by the shifter 1.5 * 2^23 (float spacing 1 in [2^23, 2^24));
    // the low bits of the shifted sum hold n
    const float shift = 12582912.0f;
    const float sh = fmaf(x, 1.44269504088896341f, shift);
    const float n = sh - shift;
    float r = fmaf(n, -0.693145751953125f, x);
    r = fmaf(n, -1.42860682030941723212e-6f, r);
    // expm1(r) = r (1 + r g(r)), g the degree-4 minimax polynomial of
    // (e^r - 1 - r)/r^2 on [-ln2/2, ln2/2] (the march's mc_expm1)
    const float cf[5] = {1.39411131385713816e-3f, 8.36317520588636398e-3f, 4.16663736104965210e-2f,
                         1.66665762662887573e-1f, 0.5f};
    float q = cf[0];
    for (int i = 1; i < 5; ++i) q = fmaf(q, r, cf[i]);
    float p = fmaf(q, r, 1.0f);
    p = p * r;
    uint32_t shb;
    memcpy(&shb, &sh, 4);
    const uint32_t bits = (shb << 23) + ((127u - 0x4B400000u) << 23);  // (n + 127) << 23
    float two_n;
    memcpy(&two_n, &bits, 4);
    return fmaf(two_n, p, two_n - 1.0f);
}

inline void p_sincos_turn(uint32_t m, float *cs, float *sn) {
    const uint32_t q = m >> 22, r = m & 0x3FFFFFu;
    const bool hi = r > 0x200000u;
    const float x = (float)(hi ? (0x400000u - r) : r) * 3.74507028e-7f;
    const float z = x * x;
    float ps = -2.50521083854417188e-8f;
    ps = fmaf(ps, z, 2.75573192239858907e-6f);
    ps = fmaf(ps, z, -1.98412698412698413e-4f);
    ps = fmaf(ps, z, 8.33333333333333333e-3f);
    ps = fmaf(ps, z, -1.66666666666666667e-1f);
    const float s = fmaf(ps * z, x, x);
    float pc = 2.08767569878680990e-9f;
    pc = fmaf(pc, z, -2.75573192239858907e-7f);
    pc = fmaf(pc, z, 2.48015873015873016e-5f);
    pc = fmaf(pc, z, -1.38888888888888889e-3f);
    pc = fmaf(pc, z, 4.16666666666666667e-2f);
    pc = fmaf(pc, z, -0.5f);
    const float c = fmaf(pc, z, 1.0f);
    const float cq = hi ? s : c, sq = hi ? c : s;
    switch (q) {
        case 0: *cs = cq; *sn = sq; break;
        case 1: *cs = -sq; *sn = cq; break;
        case 2: *cs = -cq; *sn = -sq; break;
        default: *cs = sq; *sn = -cq; break;
    }
}

// Sobol' direction numbers (Bratley-Fox recurrence) for the first four
// dimensions: primitive polynomials 1 (van der Corput), x+1, x^2+x+1,
// x^3+x+1 with initial m = (1), (1), (1,3), (1,3,1).
struct SobolDirs {
    uint32_t v[4][32];
    SobolDirs() {
        const int s_[4] = {0, 1, 2, 3};
        const int a_[4] = {0, 0, 1, 1};
        const uint32_t m0[4][3] = {{1, 0, 0}, {1, 0, 0}, {1, 3, 0}, {1, 3, 1}};
        for (int d = 0; d < 4; ++d) {
            uint32_t m[33] = {0};
            if (d == 0) {
                for (int k = 1; k <= 32; ++k) m[k] = 1;
            } else {
                const int sd = s_[d];
                for (int k = 1; k <= sd; ++k) m[k] = m0[d][k - 1];
                for (int k = sd + 1; k <= 32; ++k) {
                    uint32_t x = m[k - sd] ^ (m[k - sd] << sd);
                    for (int i = 1; i < sd; ++i)
                        if ((a_[d] >> (sd - 1 - i)) & 1) x ^= m[k - i] << i;
                    m[k] = x;
                }
            }
            for (int k = 1; k <= 32; ++k) v[d][k - 1] = m[k] << (32 - k);
        }
    }
};
static const SobolDirs g_sobol;
inline void sobol4(uint32_t idx, uint32_t out[4]) {
    uint32_t a = 0, b = 0, c = 0, d = 0;
    for (int k = 0; idx; ++k, idx >>= 1)
        if (idx & 1) { a ^= g_sobol.v[0][k]; b ^= g_sobol.v[1][k]; c ^= g_sobol.v[2][k]; d ^= g_sobol.v[3][k]; }
    out[0] = a; out[1] = b; out[2] = c; out[3] = d;
}

template <class R>
inline void p_gpos(R v, R v0, R inv, int n, int *i, R *f) {
    R p = (v - v0) * inv;
    p = std::fmin(std::fmax(p, (R)0), (R)(n - 1));
    int ii = (int)p;
    ii = std::min(ii, n - 2);
    *i = ii;
    *f = p - (R)ii;
}

template <class R> inline R FMA(R a, R b, R c) { return std::fma(a, b, c); }
template <> inline float FMA<float>(float a, float b, float c) { return fmaf(a, b, c); }

// Bins per hemisphere of the control variate's surrogate table (the device's
// kSurBins): nodes at u = m / kSurBinsO of u = sqrt(|mu|).
constexpr int kSurBinsO = 64;

// Float pairs (hi, lo) for the per-ray sums of the FP32 replay, the march's
// ff_add / ff_addf / tally_ray (this file is compiled without FMA
// contraction, so the error-free steps stay exact).
struct FPair { float h = 0.0f, l = 0.0f; };
inline FPair fp_add(FPair a, FPair b) {
    const float s = a.h + b.h;
    const float bb = s - a.h;
    float e = (a.h - (s - bb)) + (b.h - bb);
    e = e + (a.l + b.l);
    const float hi = s + e;
    return FPair{hi, e - (hi - s)};
}
inline FPair fp_addf(FPair a, float b) {
    const float s = a.h + b;
    const float bb = s - a.h;
    float e = (a.h - (s - bb)) + (b - bb);
    e = e + a.l;
    const float hi = s + e;
    return FPair{hi, e - (hi - s)};
}
inline double fp_value(FPair a) { return (double)a.h + (double)a.l; }

template <class R> inline R expm1_r(R x);
template <> inline float expm1_r<float>(float x) { return p_expm1(x); }
template <> inline double expm1_r<double>(double x) { return std::expm1(x); }

// The surrogate's straight walk (the device's cv_walk): from oW, the centre of
// layer w0, with wall-normal cosine mu > 0 in direction dW through layers of
// constant (sk[l], sI[l]), stopped beyond optical depth dtoll (the rest is
// absorbed in that layer) or at the black wall of intensity Iw.  J: the
// collected intensity; A: 1 - the transmissivity leaving layer w0 (0 if the
// walk stops inside it).
template <class R>
inline void sur_walk(const float *fw, int nw, R dtoll, const float *sk, const float *sI, int w0, R oW, R mu, int dW,
                     R Iw, R *J_out, R *A_out) {
    const R invW = (R)1 / mu;
    R J = 0, tauE = 1, tE = 0, dcum = 0, te0 = -1;
    int l = w0;
    R kS = (R)sk[w0], IS = (R)sI[w0];
    bool trunc = false;
    for (;;) {
        const R tn = (dW > 0 ? ((R)fw[l + 1] - oW) : (oW - (R)fw[l])) * invW;
        const R opt = kS * (tn - tE);
        trunc = dcum + opt > dtoll;
        if (trunc) break;
        const R a = -expm1_r<R>(-opt);
        const R ta = tauE * a;
        J = FMA<R>(ta, IS, J);
        tauE = tauE - ta;
        dcum = dcum + opt;
        tE = tn;
        if (te0 < 0) te0 = tauE;
        l += dW;
        if (l < 0 || l >= nw) break;
        kS = (R)sk[l];
        IS = (R)sI[l];
    }
    *J_out = FMA<R>(tauE, trunc ? IS : Iw, J);
    *A_out = (R)1 - (te0 < 0 ? (R)0 : te0);
}

inline float p_u24(uint32_t x) { return (float)(x >> 8) * 5.9604644775390625e-8f; }
inline float p_u24o(uint32_t x) { return ((float)(x >> 8) + 0.5f) * 5.9604644775390625e-8f; }

// -ln(u), the device's mc_neglog: u = m 2^e, m in [sqrt(1/2), sqrt(2)),
// ln m = 2 atanh((m-1)/(m+1)) by its odd series to s^11.
inline float p_neglog(float u) {
    uint32_t b;
    memcpy(&b, &u, 4);
    int e = (int)((b >> 23) & 0xffu) - 127;
    const uint32_t mb = (b & 0x7fffffu) | 0x3f800000u;
    float m;
    memcpy(&m, &mb, 4);
    if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float z = s * s;
    float p = 9.09090909090909091e-2f;
    p = fmaf(p, z, 1.11111111111111111e-1f);
    p = fmaf(p, z, 1.42857142857142857e-1f);
    p = fmaf(p, z, 2.0e-1f);
    p = fmaf(p, z, 3.33333333333333333e-1f);
    p = fmaf(p, z, 1.0f);
    const float lnm = 2.0f * s * p;
    const float fe = (float)e;
    return -fmaf(fe, 0.693145751953125f, fmaf(fe, 1.42860682030941723212e-6f, lnm));
}

// Henyey-Greenstein scattering of (sW, sA, sB), the device's hg_scatter.
template <class R>
inline void hg_scatter(R g, uint32_t uc, uint32_t um, R *sW, R *sA, R *sB) {
    const R u = (R)p_u24(uc);
    R ct;
    if (std::fabs(g) < (R)1e-6f) {
        ct = (R)1 - (R)2 * u;
    } else {
        const R tmp = ((R)1 - g * g) / ((R)1 - g + (R)2 * g * u);
        ct = ((R)1 + g * g - tmp * tmp) / ((R)2 * g);
    }
    ct = std::fmin(std::fmax(ct, (R)-1), (R)1);
    const R st = std::sqrt(std::fmax((R)0, (R)1 - ct * ct));
    float cphf, sphf;
    p_sincos_turn(um >> 8, &cphf, &sphf);
    const R cph = cphf, sph = sphf;
    const R w = *sW, a = *sA, b = *sB;
    R nw, na, nb;
    if (std::fabs(w) > (R)0.99999f) {
        na = st * cph;
        nb = st * sph;
        nw = w > 0 ? ct : -ct;
    } else {
        const R tmp = std::sqrt((R)1 - w * w);
        na = st * (a * w * cph - b * sph) / tmp + a * ct;
        nb = st * (b * w * cph + a * sph) / tmp + b * ct;
        nw = -st * cph * tmp + w * ct;
    }
    *sW = nw; *sA = na; *sB = nb;
}

template <class R>
struct Packet {
    const OrcPacketConfig &c;
    R invdT, invdX;
    long long plane, fstride;
    Packet(const OrcPacketConfig &c_) : c(c_) {
        invdT = (R)(1.0f / c.dT);
        invdX = (R)(c.nX > 1 ? 1.0f / c.dX : 1.0f);
        plane = (long long)c.na * c.nb;
        fstride = plane * c.nw;
    }
    // dense host layout: cell (w, a, b) of field f at f*fstride + w + nw*(a + na*b)
    inline long long cidx(int f, int w, int a, int b) const { return (long long)f * fstride + w + (long long)c.nw * (a + (long long)c.na * b); }
    R kfun(int koff, int ti, R ft, int xi, R fx) const {
        if (c.mode == 2) {
            const float *s = c.ktab + koff + ti * c.nX + xi;
            const R k00 = s[0], k01 = s[1], k10 = s[c.nX], k11 = s[c.nX + 1];
            const R k0 = FMA<R>(fx, k01 - k00, k00), k1 = FMA<R>(fx, k11 - k10, k10);
            return FMA<R>(ft, k1 - k0, k0);
        }
        const float *s = c.ktab + koff + ti;
        const R k0 = s[0], k1 = s[1];
        return FMA<R>(ft, k1 - k0, k0);
    }
    R ibfun(int nb, int ti, R ft) const {
        const float *s = c.ibtab + (size_t)nb * c.nT + ti;
        const R i0 = s[0], i1 = s[1];
        return FMA<R>(ft, i1 - i0, i0);
    }
    R expm1n(R x) const;  // expm1 of x <= 0
    void dirs(uint32_t x0, uint32_t x1, R *sW, R *sA, R *sB) const;

    // One work item: returns per-lane S, S2; optional trace of ray tr.
    void item(int f, int G, int p, double S[128], double S2[128], double *steps, int tr, int tmax, int32_t *rec,
              int *nrec, uint32_t *rng) const {
        // a packet is nl = 32 * cpl cells; cell l sits at (l % tile_a, l / tile_a)
        const int nl = 32 * (c.cpl > 1 ? c.cpl : 1);
        const int ta = c.tile_a, tb = nl / ta;
        const int njR = c.ea1 - c.ea0, nkR = c.eb1 - c.eb0;
        const int npa = (njR + ta - 1) / ta, npb = (nkR + tb - 1) / tb;
        const int pa = p % npa, rest = p / npa, pb = rest % npb, pw = rest / npb;
        const int w0 = c.ew0 + pw;
        int a0[128], b0[128];
        bool act[128];
        for (int l = 0; l < nl; ++l) {
            a0[l] = c.ea0 + pa * ta + l % ta;
            b0[l] = c.eb0 + pb * tb + l / ta;
            act[l] = a0[l] < c.ea1 && b0[l] < c.eb1;
            if (!act[l]) { a0[l] = c.ea0; b0[l] = c.eb0; }
            S[l] = 0; S2[l] = 0;
        }
        const int N = c.rays_per_packet ? c.rays_per_packet[G * c.rays_gstride + p] : c.rays;
        int gs = 0, K = 1;
        if (c.mode != 0) {
            int binoff = 0;
            if (c.n_tbins > 0) {
                const float T0v = c.fieldT[cidx(f, w0, a0[0], b0[0])];
                int bin = (int)rintf((T0v - c.T0) * (1.0f / c.dT));
                bin = std::min(std::max(bin, 0), c.n_tbins - 1);
                binoff = bin * c.n_groups;
            }
            gs = c.group_start[binoff + G];
            K = c.group_start[binoff + G + 1] - gs;
        }
        R Ti4[128], ft_i[128], fx_i[128];
        int ti_i[128], xi_i[128];
        for (int l = 0; l < nl; ++l) {
            const long long o = cidx(f, w0, a0[l], b0[l]);
            const R Ti = (R)c.fieldT[o];
            ti_i[l] = xi_i[l] = 0; ft_i[l] = fx_i[l] = 0; Ti4[l] = 0;
            if (c.mode == 2) p_gpos<R>((R)c.fieldX[o], (R)c.X0, invdX, c.nX, &xi_i[l], &fx_i[l]);
            if (c.mode == 0) {
                const R t2 = Ti * Ti;
                Ti4[l] = t2 * t2;
            } else {
                p_gpos<R>(Ti, (R)c.T0, invdT, c.nT, &ti_i[l], &ft_i[l]);
            }
        }
        const R oW = ((R)c.fw[w0] + (R)c.fw[w0 + 1]) * (R)0.5;
        const R Wgrey = (R)(float)(4.0 * c.kappa * 5.670373e-08);
        const R W4sig = (R)(float)(4.0 * 5.670373e-08);
        R fvown[128];
        for (int l = 0; l < nl; ++l) fvown[l] = (c.gen && c.fieldV) ? (R)c.fieldV[cidx(f, w0, a0[l], b0[l])] : (R)0;
        const float tw = c.T_west, te = c.T_east;
        const R Tw4[2] = {(R)(tw * tw * tw * tw), (R)(te * te * te * te)};
        const uint32_t k0 = (uint32_t)c.seed, k1 = (uint32_t)(c.seed >> 32);
        const int rb = tr >= 0 ? tr : 0, re = tr >= 0 ? tr + 1 : (K > 0 ? N : 0);
        const int Mb = c.sampler == 1 ? std::max(1, N / std::max(1, c.nbatch)) : 1;
        double Sb[128];
        for (int l = 0; l < nl; ++l) Sb[l] = 0.0;
        // the FP32 replay's sums as the march keeps them: float pairs
        constexpr bool kPairs = std::is_same<R, float>::value;
        FPair Sp[128], S2p[128], Sbp[128];
        for (int r = rb; r < re; ++r) {
            uint32_t x[4];
            if (c.sampler == 1) {
                const uint32_t ctr[4] = {(uint32_t)(r / Mb), (uint32_t)p, (uint32_t)G | ((uint32_t)f << 16), 0x50B01u};
                uint32_t sh[4], sb[4];
                philox(ctr, k0, k1, sh);
                sobol4((uint32_t)(r % Mb), sb);
                for (int d = 0; d < 4; ++d) x[d] = sb[d] ^ sh[d];
            } else {
                const uint32_t ctr[4] = {(uint32_t)r, (uint32_t)p, (uint32_t)G | ((uint32_t)f << 16), 0u};
                philox(ctr, k0, k1, x);
            }
            if (rng) memcpy(rng, x, sizeof x);
            R sW, sA, sB;
            dirs(x[0], x[1], &sW, &sA, &sB);
            int nbnd = 0, koff = 0;
            R We = 0;
            if (c.mode != 0) {
                const int j = (int)(((uint64_t)x[2] * (uint64_t)K) >> 32);
                int e = gs + j;
                const float u = (float)(x[3] >> 8) * 5.9604644775390625e-8f;
                if (!(u < c.prob[e])) e = gs + c.alias[e];
                nbnd = c.band[e];
                koff = (nbnd * c.nq + c.gq[e]) * c.nT * c.nX;
                We = (R)c.W[e];
            }
            // general medium: particle coefficients of the band
            R pab = 0, psc = 0;
            if (c.gen && c.part) { pab = (R)c.part[2 * nbnd]; psc = (R)c.part[2 * nbnd + 1]; }
            R wk[128], Ii[128], tau[128], D[128];
            for (int l = 0; l < nl; ++l) {
                if (c.mode == 0) {
                    Ii[l] = Ti4[l];
                    wk[l] = c.gen ? W4sig * FMA<R>(fvown[l], pab, (R)c.kappa) : Wgrey;
                } else {
                    R ki = kfun(koff, ti_i[l], ft_i[l], xi_i[l], fx_i[l]);
                    if (c.gen) ki = FMA<R>(fvown[l], pab, ki);
                    Ii[l] = ibfun(nbnd, ti_i[l], ft_i[l]);
                    wk[l] = We * ki;
                }
                tau[l] = act[l] ? (R)1 : (R)0;
                D[l] = 0;
            }
            // surrogate: the straight flight through the layer-mean medium,
            // advanced once per layer, stopped beyond optical depth ln(1/toll)
            const int sid = c.mode != 0 ? koff / (c.nT * c.nX) : 0;
            const int nsamp = c.mode != 0 ? c.nbands * c.nq : 1;
            const size_t sbase = ((size_t)f * nsamp + sid) * c.nw;
            R Jbar = 0, Aown = 0;
            if (c.cv) {
                if (c.sur_tab) {  // the march's table read: linear in sqrt(|sW|)
                    const float x = std::sqrt(std::fabs((float)sW)) * (float)kSurBinsO;
                    const int m = std::min((int)x, kSurBinsO - 1);
                    const float r = x - (float)m;
                    const float *e = c.sur_tab + (((sbase + w0) * 2 + (sW > 0 ? 1 : 0)) * kSurBinsO + m) * 4;
                    Jbar = FMA<R>((R)r, (R)e[1], (R)e[0]);
                    Aown = FMA<R>((R)r, (R)e[3], (R)e[2]);
                } else {
                    const int side = sW > 0 ? 1 : 0;
                    const R Iws = c.mode == 0 ? Tw4[side] : (R)c.ibw[side * c.nbands + nbnd];
                    sur_walk<R>(c.fw, c.nw, (R)(float)(-std::log((double)c.toll)), c.sur_k + sbase,
                                c.sur_I + sbase, w0, oW, std::fabs(sW), sW > 0 ? 1 : -1, Iws, &Jbar, &Aown);
                }
            }
            // warp-uniform DDA from (pw0, fa0, fb0)
            R pw0 = oW, fa0 = (R)0.5, fb0 = (R)0.5, offA = (R)0.5, offB = (R)0.5;
            R invW, invA, invB, tW, dtA, dtB, tA, tB;
            int dW, dA, dB, nA, nB;
            int cw = w0, stepn = 0;
            auto dda_init = [&]() {
                invW = (R)1 / std::fabs(sW); invA = (R)1 / std::fabs(sA); invB = (R)1 / std::fabs(sB);
                dW = sW > 0 ? 1 : -1; dA = sA > 0 ? 1 : -1; dB = sB > 0 ? 1 : -1;
                tW = (dW > 0 ? ((R)c.fw[cw + 1] - pw0) : (pw0 - (R)c.fw[cw])) * invW;
                dtA = (R)c.da * invA; dtB = (R)c.db * invB;
                if (c.gen) {
                    offA = dA > 0 ? (R)1 - fa0 : fa0;
                    offB = dB > 0 ? (R)1 - fb0 : fb0;
                }
                tA = offA * dtA; tB = offB * dtB;
                nA = 0; nB = 0;
            };
            dda_init();
            int ca[128], cb[128];
            for (int l = 0; l < nl; ++l) { ca[l] = a0[l]; cb[l] = b0[l]; }
            R t = 0;
            // scattering events
            uint32_t ev = 0, evx[4] = {0, 0, 0, 0};
            auto draw = [&]() {
                const uint32_t ctr[4] = {(uint32_t)r, (uint32_t)p, (uint32_t)G | ((uint32_t)f << 16), 0x5CA70000u + ev};
                philox(ctr, k0, k1, evx);
                ++ev;
            };
            const R INF = std::numeric_limits<R>::infinity();
            R sigbar = 0, tcol = INF;
            if (c.gen) {
                sigbar = (R)c.fv_max * psc;
                if (sigbar > 0) { draw(); tcol = (R)p_neglog(p_u24o(evx[0])) / sigbar; }
            }
            auto field_k = [&](int l, long long o, R *gj) -> R {
                R kj;
                if (c.mode == 0) {
                    const R Tj = (R)c.fieldT[o];
                    const R t2 = Tj * Tj;
                    *gj = Ti4[l] - t2 * t2;
                    kj = (R)c.kappa;
                } else {
                    int tj, xj = 0;
                    R ftj, fxj = 0;
                    if (c.mode == 2) p_gpos<R>((R)c.fieldX[o], (R)c.X0, invdX, c.nX, &xj, &fxj);
                    p_gpos<R>((R)c.fieldT[o], (R)c.T0, invdT, c.nT, &tj, &ftj);
                    kj = kfun(koff, tj, ftj, xj, fxj);
                    *gj = Ii[l] - ibfun(nbnd, tj, ftj);
                }
                if (c.gen && c.fieldV) kj = FMA<R>((R)c.fieldV[o], pab, kj);
                return kj;
            };
            auto shift_point = [&]() {  // fractional offsets at parameter t of the current segment
                const R ta_ = t / dtA, tb_ = t / dtB;
                fa0 = dA > 0 ? fa0 + (ta_ - (R)nA) : fa0 - (ta_ - (R)nA);
                fb0 = dB > 0 ? fb0 + (tb_ - (R)nB) : fb0 - (tb_ - (R)nB);
                fa0 = std::fmin(std::fmax(fa0, (R)0), (R)1);
                fb0 = std::fmin(std::fmax(fb0, (R)0), (R)1);
            };
            for (;;) {
                int axis;
                R tn;
                if (tW <= tA && tW <= tB) { axis = 0; tn = tW; }
                else if (tA <= tB) { axis = 1; tn = tA; }
                else { axis = 2; tn = tB; }
                if (c.gen && tcol < tn) { axis = 3; tn = tcol; }
                const R ds = tn - t;
                for (int l = 0; l < nl; ++l) {
                    if (!(tau[l] > 0)) continue;
                    *steps += 1;
                    const long long o = cidx(f, cw, ca[l], cb[l]);
                    R gj;
                    const R kj = field_k(l, o, &gj);
                    const R alpha = -expm1n(-(kj * ds));
                    const R tal = tau[l] * alpha;
                    D[l] = FMA<R>(tal, gj, D[l]);
                    tau[l] = tau[l] - tal;
                    if (tau[l] < (R)c.toll) { D[l] = FMA<R>(tau[l], gj, D[l]); tau[l] = 0; }
                }
                if (rec && stepn < tmax) {
                    int32_t *q = rec + 6 * stepn;
                    q[0] = cw; q[1] = dA * nA; q[2] = dB * nB; q[3] = axis;
                    const float dsf = (float)ds, tf = (float)tau[0];
                    memcpy(&q[4], &dsf, 4);
                    memcpy(&q[5], &tf, 4);
                }
                t = tn;
                ++stepn;
                if (axis == 0) {
                    if (cw + dW < 0 || cw + dW >= c.nw) {
                        const int side = cw + dW < 0 ? 0 : 1;
                        const R Iw = c.mode == 0 ? Tw4[side] : (R)c.ibw[side * c.nbands + nbnd];
                        if (c.gen) {
                            const R eps = (R)c.eps[side];
                            bool any = false;
                            for (int l = 0; l < nl; ++l) {
                                if (tau[l] > 0) {
                                    const R gw = Ii[l] - Iw;
                                    D[l] = FMA<R>(tau[l] * eps, gw, D[l]);
                                    tau[l] = eps >= (R)1 ? (R)0 : tau[l] * ((R)1 - eps);
                                    if (tau[l] > 0 && tau[l] < (R)c.toll) { D[l] = FMA<R>(tau[l], gw, D[l]); tau[l] = 0; }
                                }
                                any = any || tau[l] > 0;
                            }
                            if (!any) break;
                            shift_point();
                            pw0 = side == 0 ? (R)c.fw[0] : (R)c.fw[c.nw];
                            draw();
                            const R cmu = std::sqrt((R)p_u24(evx[2]));
                            const R smu = std::sqrt(std::fmax((R)0, (R)1 - cmu * cmu));
                            float cpf, spf;
                            p_sincos_turn(evx[3] >> 8, &cpf, &spf);
                            sW = side == 0 ? cmu : -cmu;
                            sA = smu * (R)cpf;
                            sB = smu * (R)spf;
                            dda_init();
                            t = 0;
                            if (sigbar > 0) { draw(); tcol = (R)p_neglog(p_u24o(evx[0])) / sigbar; }
                            if (stepn >= c.max_steps) break;
                            continue;
                        }
                        for (int l = 0; l < nl; ++l) {
                            if (!(tau[l] > 0)) continue;
                            D[l] = FMA<R>(tau[l], Ii[l] - Iw, D[l]);
                            tau[l] = 0;
                        }
                        break;
                    }
                    cw += dW;
                    tW = (dW > 0 ? ((R)c.fw[cw + 1] - pw0) : (pw0 - (R)c.fw[cw])) * invW;
                } else if (axis == 1) {
                    ++nA;
                    tA = ((R)nA + offA) * dtA;
                    for (int l = 0; l < nl; ++l) { ca[l] += dA; if (ca[l] == c.na) ca[l] = 0; else if (ca[l] < 0) ca[l] = c.na - 1; }
                } else if (axis == 2) {
                    ++nB;
                    tB = ((R)nB + offB) * dtB;
                    for (int l = 0; l < nl; ++l) { cb[l] += dB; if (cb[l] == c.nb) cb[l] = 0; else if (cb[l] < 0) cb[l] = c.nb - 1; }
                } else {
                    // tentative collision: shared decision, per-cell weights;
                    // q is the device's sum: each lane adds its cells l, l + 32,
                    // ... in order, then the butterfly (xor 16, 8, 4, 2, 1)
                    R pl[128], ps[32], pc[32];
                    for (int l = 0; l < nl; ++l) {
                        const R fvl = c.fieldV ? (R)c.fieldV[cidx(f, cw, ca[l], cb[l])] : (R)0;
                        pl[l] = tau[l] > 0 ? std::fmin((R)1, fvl * psc / sigbar) : (R)0;
                    }
                    for (int l = 0; l < 32; ++l) {
                        ps[l] = pl[l];
                        pc[l] = tau[l] > 0 ? (R)1 : (R)0;
                        for (int k = l + 32; k < nl; k += 32) {
                            ps[l] = ps[l] + pl[k];
                            pc[l] = pc[l] + (tau[k] > 0 ? (R)1 : (R)0);
                        }
                    }
                    for (int o = 16; o > 0; o >>= 1) {
                        R ns[32], nc[32];
                        for (int l = 0; l < 32; ++l) { ns[l] = ps[l] + ps[l ^ o]; nc[l] = pc[l] + pc[l ^ o]; }
                        for (int l = 0; l < 32; ++l) { ps[l] = ns[l]; pc[l] = nc[l]; }
                    }
                    const R q = pc[0] > 0 ? ps[0] / pc[0] : (R)0;
                    if ((R)p_u24(evx[1]) < q) {
                        for (int l = 0; l < nl; ++l)
                            if (tau[l] > 0) tau[l] = tau[l] * (pl[l] / q);
                        shift_point();
                        pw0 = std::fmin(std::fmax(FMA<R>(sW, t, pw0), (R)c.fw[cw]), (R)c.fw[cw + 1]);
                        hg_scatter<R>((R)c.hg_g, evx[2], evx[3], &sW, &sA, &sB);
                        dda_init();
                        t = 0;
                    } else {
                        for (int l = 0; l < nl; ++l)
                            if (tau[l] > 0) tau[l] = tau[l] * (((R)1 - pl[l]) / ((R)1 - q));
                    }
                    draw();
                    tcol = t + (R)p_neglog(p_u24o(evx[0])) / sigbar;
                }
                bool any = false;
                for (int l = 0; l < nl; ++l) any = any || (tau[l] > 0);
                if (!any) break;
                if (stepn >= (c.mg_levels > 1 ? c.mg_steps : c.max_steps)) break;
            }
            if (c.mg_levels > 1) {
                // coarse grids: per-lane position-update march in lockstep
                bool any = false;
                for (int l = 0; l < nl; ++l) any = any || (tau[l] > 0);
                if (any) {
                    const R ua = t / dtA - (R)nA, ub = t / dtB - (R)nB;
                    const R fa = std::fmin(std::fmax(dA > 0 ? (R)0.5 + ua : (R)0.5 - ua, (R)0), (R)1);
                    const R fb = std::fmin(std::fmax(dB > 0 ? (R)0.5 + ub : (R)0.5 - ub, (R)0), (R)1);
                    R xp[128], yp[128], zp[128];
                    int ic[128], jc[128], kc[128];
                    for (int l = 0; l < nl; ++l) {
                        xp[l] = FMA<R>(sW, t, oW);
                        yp[l] = ((R)ca[l] + fa) * (R)c.da;
                        zp[l] = ((R)cb[l] + fb) * (R)c.db;
                        ic[l] = cw; jc[l] = ca[l]; kc[l] = cb[l];
                    }
                    const R isx = (R)1 / sW, isy = (R)1 / sA, isz = (R)1 / sB;
                    for (int lv = 1; lv < c.mg_levels; ++lv) {
                        const int nwL = c.nw >> lv, naL = c.na >> lv, nbL = c.nb >> lv;
                        const float *fwL = c.mgfw + c.mg_fwoff[lv];
                        const R daL = (R)c.mg_da[lv], dbL = (R)c.mg_db[lv];
                        const float *TL = c.mgT + c.mg_off[lv] + (long long)f * nwL * naL * nbL;
                        const int cap = (lv == c.mg_levels - 1) ? c.max_steps : c.mg_steps;
                        for (int l = 0; l < nl; ++l) { ic[l] >>= 1; jc[l] >>= 1; kc[l] >>= 1; }
                        int counter = 0;
                        for (;;) {
                            bool go = false;
                            for (int l = 0; l < nl; ++l) go = go || (tau[l] > 0 && counter < cap);
                            if (!go) break;
                            R dsr0 = 0;  // lane 0's segment this iteration (0 when it idles)
                            for (int l = 0; l < nl; ++l) {
                                if (!(tau[l] > 0 && counter < cap)) continue;
                                *steps += 1;
                                const R fx = (R)fwL[dW > 0 ? ic[l] + 1 : ic[l]];
                                const R fy = (R)(float)(dA > 0 ? jc[l] + 1 : jc[l]) * daL;
                                const R fz = (R)(float)(dB > 0 ? kc[l] + 1 : kc[l]) * dbL;
                                const R dsx = sW != 0 ? (fx - xp[l]) * isx : INF;
                                const R dsy = sA != 0 ? (fy - yp[l]) * isy : INF;
                                const R dsz = sB != 0 ? (fz - zp[l]) * isz : INF;
                                const R Tc = (R)TL[((long long)ic[l] * nbL + kc[l]) * naL + jc[l]];
                                R kj, gj;
                                if (c.mode == 0) {
                                    const R t2 = Tc * Tc;
                                    gj = Ti4[l] - t2 * t2;
                                    kj = (R)c.kappa;
                                } else {
                                    int tj;
                                    R ftj;
                                    p_gpos<R>(Tc, (R)c.T0, invdT, c.nT, &tj, &ftj);
                                    kj = kfun(koff, tj, ftj, 0, 0);
                                    gj = Ii[l] - ibfun(nbnd, tj, ftj);
                                }
                                R dmin = dsx;
                                if (dmin > dsy) dmin = dsy;
                                if (dmin > dsz) dmin = dsz;
                                const R ds = std::fmax(dmin, (R)0);
                                if (l == 0) dsr0 = ds;
                                xp[l] = (dmin == dsx) ? fx : FMA<R>(ds, sW, xp[l]);
                                yp[l] = (dmin == dsy) ? fy : FMA<R>(ds, sA, yp[l]);
                                zp[l] = (dmin == dsz) ? fz : FMA<R>(ds, sB, zp[l]);
                                const R alpha = -expm1n(-(kj * ds));
                                const R tal = tau[l] * alpha;
                                D[l] = FMA<R>(tal, gj, D[l]);
                                tau[l] = tau[l] - tal;
                                if (tau[l] < (R)c.toll) { D[l] = FMA<R>(tau[l], gj, D[l]); tau[l] = 0; }
                                int axis;
                                if (dsx < dsy) axis = (dsx < dsz) ? 0 : 2;
                                else axis = (dsy < dsz) ? 1 : 2;
                                if (axis == 0) {
                                    ic[l] += dW;
                                    if (ic[l] < 0 || ic[l] >= nwL) {
                                        const int side = ic[l] < 0 ? 0 : 1;
                                        const R Iw = c.mode == 0 ? Tw4[side] : (R)c.ibw[side * c.nbands + nbnd];
                                        if (tau[l] > 0) D[l] = FMA<R>(tau[l], Ii[l] - Iw, D[l]);
                                        tau[l] = 0;
                                        ic[l] = ic[l] < 0 ? 0 : nwL - 1;
                                    }
                                } else if (axis == 1) {
                                    jc[l] += dA;
                                    if (jc[l] >= naL) { jc[l] = 0; yp[l] = 0; } else if (jc[l] < 0) { jc[l] = naL - 1; yp[l] = (R)c.Ly; }
                                } else {
                                    kc[l] += dB;
                                    if (kc[l] >= nbL) { kc[l] = 0; zp[l] = 0; } else if (kc[l] < 0) { kc[l] = nbL - 1; zp[l] = (R)c.Lz; }
                                }
                            }
                            if (rec && stepn < tmax) {  // lane 0, every iteration
                                int32_t *q = rec + 6 * stepn;
                                q[0] = ic[0]; q[1] = jc[0]; q[2] = kc[0]; q[3] = 16 + lv;
                                const float dsf = (float)dsr0, tf = (float)tau[0];
                                memcpy(&q[4], &dsf, 4);
                                memcpy(&q[5], &tf, 4);
                            }
                            ++counter;
                            ++stepn;
                        }
                    }
                }
            }
            if (nrec) *nrec = stepn;
            for (int l = 0; l < nl; ++l) {
                if (!act[l]) continue;
                R X = wk[l] * D[l];
                if (c.cv) {
                    const int nG = c.mode == 0 ? 1 : c.n_groups;
                    const int niR = c.ew1 - c.ew0, njR = c.ea1 - c.ea0, nkR = c.eb1 - c.eb0;
                    const long long rc = (long long)niR * njR * nkR;
                    R ba = 1, bb = -1;
                    if (c.beta) {
                        const float *bp = c.beta + 2 * (((long long)f * nG + G) * rc + (w0 - c.ew0) +
                                                         (long long)niR * ((a0[l] - c.ea0) + (long long)njR * (b0[l] - c.eb0)));
                        ba = (R)bp[0];
                        bb = (R)bp[1];
                    }
                    const R Iw0 = (R)c.sur_I[sbase + w0];
                    const R Ya = wk[l] * (Ii[l] - Jbar);
                    const R Yb = wk[l] * (Aown * (Ii[l] - Iw0));
                    if (c.moments) {
                        const long long tc = ((long long)(w0 - c.ew0) * nkR + (b0[l] - c.eb0)) * njR + (a0[l] - c.ea0);
                        double *mo = c.moments + 9 * (((long long)f * nG + G) * rc + tc);
                        const double xd = (double)X, ya = (double)Ya, yb = (double)Yb;
                        mo[0] += xd; mo[1] += ya; mo[2] += yb;
                        mo[3] = std::fma(xd, xd, mo[3]); mo[4] = std::fma(ya, ya, mo[4]); mo[5] = std::fma(yb, yb, mo[5]);
                        mo[6] = std::fma(xd, ya, mo[6]); mo[7] = std::fma(xd, yb, mo[7]); mo[8] = std::fma(ya, yb, mo[8]);
                    }
                    X = X - ba * Ya;
                    X = X - bb * Yb;
                }
                if constexpr (kPairs) {
                    const float Xf = (float)X;
                    Sp[l] = fp_addf(Sp[l], Xf);
                    if (c.sampler == 1) {
                        const FPair Sbl = fp_addf(Sbp[l], Xf);
                        if (r % Mb == Mb - 1) {
                            const float Mf = (float)Mb;
                            const float q = Sbl.h / Mf;
                            const float ql = (fmaf(-q, Mf, Sbl.h) + Sbl.l) / Mf;
                            const float pq = q * q;
                            S2p[l] = fp_add(S2p[l], FPair{pq, fmaf(q, q, -pq) + 2.0f * (q * ql)});
                            Sbp[l] = FPair{};
                        } else {
                            Sbp[l] = Sbl;
                        }
                    } else {
                        const float pq = Xf * Xf;
                        S2p[l] = fp_add(S2p[l], FPair{pq, fmaf(Xf, Xf, -pq)});
                    }
                    continue;
                }
                const double Xd = (double)X;
                S[l] += Xd;
                if (c.sampler == 1) {
                    Sb[l] += Xd;
                    if (r % Mb == Mb - 1) {
                        const double mb = Sb[l] / Mb;
                        S2[l] = std::fma(mb, mb, S2[l]);
                        Sb[l] = 0.0;
                    }
                } else {
                    S2[l] = std::fma(Xd, Xd, S2[l]);
                }
            }
        }
        if constexpr (kPairs)
            for (int l = 0; l < nl; ++l) { S[l] = fp_value(Sp[l]); S2[l] = fp_value(S2p[l]); }
    }
};

template <> float Packet<float>::expm1n(float x) const { return p_expm1(x); }
template <> double Packet<double>::expm1n(double x) const { return std::expm1(x); }
template <> void Packet<float>::dirs(uint32_t x0, uint32_t x1, float *sW, float *sA, float *sB) const {
    const float mu = fmaf((float)(x1 >> 8), -1.1920928955078125e-7f, 1.0f);
    const float st = sqrtf(std::fmax(0.0f, fmaf(-mu, mu, 1.0f)));
    float cph, sph;
    p_sincos_turn(x0 >> 8, &cph, &sph);
    *sW = mu; *sA = st * cph; *sB = st * sph;
}
template <> void Packet<double>::dirs(uint32_t x0, uint32_t x1, double *sW, double *sA, double *sB) const {
    const double mu = 1.0 - (double)(x1 >> 8) * 1.1920928955078125e-7;
    const double st = std::sqrt(std::max(0.0, 1.0 - mu * mu));
    const double ph = 2.0 * 3.14159265358979323846 * (double)(x0 >> 8) * 5.9604644775390625e-8;
    *sW = mu; *sA = st * std::cos(ph); *sB = st * std::sin(ph);
}

}  // namespace

extern "C" {

// The march's expm1 (x <= 0) on n values: the accuracy tests call it.
void orc_expm1n(const float *x, float *out, long long n) {
    for (long long i = 0; i < n; ++i) out[i] = p_expm1(x[i]);
}

// Tally [f][G][iR][kR][jR][2] (sum X, sum X^2) exactly as the device stores it.
int orc_packet_mc(const OrcPacketConfig *c, int nthreads, double *tally, double *steps_out) {
    if (!c || c->tile_a < 1 || 32 % c->tile_a || c->cpl < 0 || c->cpl > 4) return 1;
    if (c->cpl > 1 && c->mg_levels > 1) return 1;  // the multigrid march runs 32-cell packets
    const int nl = 32 * (c->cpl > 1 ? c->cpl : 1);
    const int ta = c->tile_a, tb = nl / ta;
    const int niR = c->ew1 - c->ew0, njR = c->ea1 - c->ea0, nkR = c->eb1 - c->eb0;
    const int npa = (njR + ta - 1) / ta, npb = (nkR + tb - 1) / tb;
    const int step = c->pw_step > 1 ? c->pw_step : 1;
    const int np = npa * npb * ((niR + step - 1) / step);
    const int nG = c->mode == 0 ? 1 : c->n_groups;
    const long long items = (long long)c->nfields * nG * np;
    const long long rc = (long long)niR * njR * nkR;
    double steps = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : steps)
    for (long long it = 0; it < items; ++it) {
        // packet of the region (layers strided by pw_step) and its natural
        // index, which keys its rays and ray counts as in an unstrided run
        const int ps = (int)(it % np);
        const int p = ps % (npa * npb) + (ps / (npa * npb)) * step * npa * npb;
        const long long fg = it / np;
        const int G = (int)(fg % nG), f = (int)(fg / nG);
        double S[128], S2[128], st = 0;
        if (c->use_double) Packet<double>(*c).item(f, G, p, S, S2, &st, -1, 0, nullptr, nullptr, nullptr);
        else Packet<float>(*c).item(f, G, p, S, S2, &st, -1, 0, nullptr, nullptr, nullptr);
        steps += st;
        const int pa = p % npa, rest = p / npa, pb = rest % npb, pw = rest / npb;
        for (int l = 0; l < nl; ++l) {
            const int a = c->ea0 + pa * ta + l % ta, b = c->eb0 + pb * tb + l / ta;
            if (a >= c->ea1 || b >= c->eb1) continue;
            const long long tc = ((long long)pw * nkR + (b - c->eb0)) * njR + (a - c->ea0);
            tally[2 * (fg * rc + tc)] = S[l];
            tally[2 * (fg * rc + tc) + 1] = S2[l];
        }
    }
    if (steps_out) *steps_out = steps;
    return 0;
}

// The control variate's surrogate table (the device's cv_table_kernel), in
// FP32: per (field, sample) and hemisphere h (0: towards the west wall, 1:
// east) and node mu = (m / kSurBinsO)^2, m = 0 .. kSurBinsO (m = 0 at mu =
// 2^-30), one sweep from the far black wall (grey: T_wall^4, tables: ibw)
// through the layer-mean medium (sur_k, sur_I) gives every layer's
// straight flight from its centre:
//   J_l = F + e1h (F - Ib_l), A_l = -e1h, then F <- F + e1 (F - Ib_l),
// e1h = expm1(-k_l h_l / mu) over the own half layer towards the wall,
// e1 = expm1(-k_l (f_{l+1} - f_l) / mu) over the whole layer, F starting at
// the wall's intensity (F: the intensity collected by a ray entering the
// layer from the side away from the wall).  Each bin m stored as (J0, dJ,
// A0, dA) = (J(m), J(m+1) - J(m), A(m), A(m+1) - A(m)).
// tab: [f][sample][nw][2][kSurBinsO][4].  JA (or NULL): [f][sample][nw][2]
// the exact means of the interpolant over mu uniform on [-1, 1]: with u =
// sqrt(|mu|) of density 2u, bin m weighs ((2m+1) J0 + (m + 2/3) dJ) /
// kSurBinsO^2 per hemisphere, the hemispheres 1/2 each.
int orc_cv_table(const OrcPacketConfig *c, float *tab, double *JA) {
    if (!c || !c->sur_k || !c->sur_I || !tab) return 1;
    const int nw = c->nw, nsamp = c->mode == 0 ? 1 : c->nbands * c->nq, NB = kSurBinsO;
    const float tw = c->T_west, te = c->T_east;
    const float Tw4[2] = {tw * tw * tw * tw, te * te * te * te};
#pragma omp parallel for schedule(dynamic, 4)
    for (long long fs = 0; fs < (long long)c->nfields * nsamp; ++fs) {
        const int band = c->mode == 0 ? 0 : (int)(fs % nsamp) / c->nq;
        const float *sk = c->sur_k + (size_t)fs * nw, *sI = c->sur_I + (size_t)fs * nw;
        std::vector<float> J((size_t)nw * 2 * (NB + 1)), A(J.size());  // [l][h][m]
        for (int h = 0; h < 2; ++h)
            for (int m = 0; m <= NB; ++m) {
                const float u = (float)m * (1.0f / (float)NB);
                const float mu = m ? u * u : 9.31322574615478516e-10f;
                const float invmu = 1.0f / mu;
                float F = c->mode == 0 ? Tw4[h] : c->ibw[h * c->nbands + band];
                for (int step = 0; step < nw; ++step) {
                    const int l = h ? nw - 1 - step : step;
                    const float f0 = c->fw[l], f1 = c->fw[l + 1];
                    const float o = (f0 + f1) * 0.5f;
                    const float half = h ? (f1 - o) * invmu : (o - f0) * invmu;
                    const float e1h = p_expm1(-(sk[l] * half));
                    J[((size_t)l * 2 + h) * (NB + 1) + m] = fmaf(e1h, F - sI[l], F);
                    A[((size_t)l * 2 + h) * (NB + 1) + m] = -e1h;
                    const float e1 = p_expm1(-(sk[l] * ((f1 - f0) * invmu)));
                    F = fmaf(e1, F - sI[l], F);
                }
            }
        for (int l = 0; l < nw; ++l) {
            float *row = tab + ((size_t)fs * nw + l) * 2 * NB * 4;
            double eJ = 0, eA = 0;
            for (int h = 0; h < 2; ++h) {
                const float *Jr = &J[((size_t)l * 2 + h) * (NB + 1)], *Ar = &A[((size_t)l * 2 + h) * (NB + 1)];
                for (int m = 0; m < NB; ++m) {
                    float *e = row + (h * NB + m) * 4;
                    e[0] = Jr[m];
                    e[1] = Jr[m + 1] - Jr[m];
                    e[2] = Ar[m];
                    e[3] = Ar[m + 1] - Ar[m];
                    const double c0 = (double)(2 * m + 1), c1 = (double)m + 2.0 / 3.0;
                    eJ += c0 * (double)e[0] + c1 * (double)e[1];
                    eA += c0 * (double)e[2] + c1 * (double)e[3];
                }
            }
            if (JA) {
                const double sc = 0.5 / ((double)NB * (double)NB);
                JA[2 * ((size_t)fs * nw + l)] = eJ * sc;
                JA[2 * ((size_t)fs * nw + l) + 1] = eA * sc;
            }
        }
    }
    return 0;
}

// Exact means of the control variate of the packet replay (cv = 1), in FP64,
// for every region cell and band group: E[Y_a] = sum_s C_s k_s(T_i, x_i)
// (Ib_s(T_i) - Jhat_s(l)) and E[Y_b] = sum_s C_s k_s(T_i, x_i) Ahat_s(l)
// (Ib_s(T_i) - Ibar_s(l)) over the group's samples s (grp_start / sid / C),
// with Jhat_s(l) and Ahat_s(l) the direction averages of the surrogate's
// collected intensity and own-layer absorptance: the straight flight from the
// centre of layer l through the layer-mean medium (sur_k, sur_I), stopped
// beyond optical depth ln(1/toll) or at the black walls (ibw), integrated over
// mu on both hemispheres with the caller's quadrature (mu, w on [0, 1]).
// muY: [f][G][tc][2] in tally order (with pw_step > 1 only the replay's
// layers are written).  Table models (mode 1, 2) only.
int orc_cv_mean(const OrcPacketConfig *c, const int *grp_start, const int *sid, const double *C, const double *mu,
                const double *wq, int nquad, int nthreads, double *muY) {
    if (!c || c->mode == 0 || !c->sur_k || !c->sur_I) return 1;
    const int nw = c->nw, nsamp = c->nbands * c->nq, nG = c->n_groups;
    const int niR = c->ew1 - c->ew0, njR = c->ea1 - c->ea0, nkR = c->eb1 - c->eb0;
    const long long rc = (long long)niR * njR * nkR;
    const double dtoll = (double)(float)(-std::log((double)c->toll));
    const int step = c->pw_step > 1 ? c->pw_step : 1;
    std::vector<double> J((size_t)c->nfields * nsamp * nw), A(J.size());
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 4)
    for (long long fs = 0; fs < (long long)c->nfields * nsamp; ++fs) {
        const int s_ = (int)(fs % nsamp), b = s_ / c->nq;
        const float *sk = c->sur_k + (size_t)fs * nw, *sI = c->sur_I + (size_t)fs * nw;
        for (int l = c->ew0; l < c->ew1; l += step) {  // the region's (solved) layers
            const double o = 0.5 * ((double)c->fw[l] + (double)c->fw[l + 1]);
            double acc = 0, accA = 0;
            for (int d = -1; d <= 1; d += 2) {
                const double Iw = c->ibw[(d < 0 ? 0 : 1) * c->nbands + b];
                for (int q = 0; q < nquad; ++q) {
                    const double m = mu[q];
                    double tau = 1, Jv = 0, t0 = 0, dcum = 0;
                    int i = l;
                    double seg = d > 0 ? ((double)c->fw[l + 1] - o) : (o - (double)c->fw[l]);
                    for (;;) {
                        const double opt = (double)sk[i] * seg / m;
                        if (dcum + opt > dtoll) { Jv += tau * (double)sI[i]; break; }
                        const double a = -std::expm1(-opt);
                        Jv += tau * a * (double)sI[i];
                        tau -= tau * a;
                        dcum += opt;
                        if (i == l) t0 = tau;
                        i += d;
                        if (i < 0 || i >= nw) { Jv += tau * Iw; break; }
                        seg = (double)c->fw[i + 1] - (double)c->fw[i];
                    }
                    acc += wq[q] * Jv;
                    accA += wq[q] * (1.0 - t0);
                }
            }
            J[(size_t)fs * nw + l] = 0.5 * acc;
            A[(size_t)fs * nw + l] = 0.5 * accA;
        }
    }
    const double invdT = 1.0 / (double)c->dT, invdX = c->nX > 1 ? 1.0 / (double)c->dX : 1.0;
#pragma omp parallel for schedule(static)
    for (long long fc = 0; fc < (long long)c->nfields * rc; ++fc) {
        const int f = (int)(fc / rc);
        const long long tc = fc % rc;
        const int a = (int)(tc % njR), b = (int)((tc / njR) % nkR), w = (int)(tc / ((long long)njR * nkR));
        if (w % step) continue;  // a layer the replay skips
        const int wi = c->ew0 + w, ai = c->ea0 + a, bi = c->eb0 + b;
        const long long o = (long long)f * nw * c->na * c->nb + wi + (long long)nw * (ai + (long long)c->na * bi);
        int ti = 0, xi = 0;
        double ft = 0, fx = 0;
        p_gpos<double>((double)c->fieldT[o], (double)c->T0, invdT, c->nT, &ti, &ft);
        if (c->mode == 2) p_gpos<double>((double)c->fieldX[o], (double)c->X0, invdX, c->nX, &xi, &fx);
        for (int G = 0; G < nG; ++G) {
            double ea = 0, eb = 0;
            for (int e = grp_start[G]; e < grp_start[G + 1]; ++e) {
                const int s_ = sid[e], band = s_ / c->nq;
                const float *kt = c->ktab + (size_t)s_ * c->nT * c->nX + (size_t)ti * c->nX + xi;
                double k;
                if (c->mode == 2) {
                    const double k0 = (double)kt[0] + fx * ((double)kt[1] - (double)kt[0]);
                    const double k1 = (double)kt[c->nX] + fx * ((double)kt[c->nX + 1] - (double)kt[c->nX]);
                    k = k0 + ft * (k1 - k0);
                } else {
                    k = (double)kt[0] + ft * ((double)kt[1] - (double)kt[0]);
                }
                const float *ib = c->ibtab + (size_t)band * c->nT + ti;
                const double Ib = (double)ib[0] + ft * ((double)ib[1] - (double)ib[0]);
                const size_t js = ((size_t)f * nsamp + s_) * nw + wi;
                ea += C[e] * k * (Ib - J[js]);
                eb += C[e] * k * A[js] * (Ib - (double)c->sur_I[js]);
            }
            double *out = muY + 2 * (((long long)f * nG + G) * rc + tc);
            out[0] = ea;
            out[1] = eb;
        }
    }
    return 0;
}

// Correlated-k distribution of line-by-line spectra (distr/correlatedK.cpp:
// 145-300, correlatedKT, and k_avg of distr/calc_prob.cpp:17-119): per
// (spectrum s, band b) the band's smallest and largest k, n_pwrk bins uniform
// in k^0.1 (pwr = 0.1), the interval between points h-1 and h at its midpoint
// k in bin MAX(0, (int)((k^0.1 - kmin^0.1) / step + 1)), the spectral
// fraction of a bin = its interval count x dwv / band width (uniform spectra),
// g(h) = 1 - sum of the fractions of bins h+1 .. n_pwrk-1, bin values
// k(h) = (e(h) + e(h+1)) / 2 with e(h) = (kmin^0.1 + h step)^10 (ten-fold
// products), k at each quadrature point by linear interpolation between the
// first bins with g(h+1) >= g_q, and the band mean sum_h k(h) fraction(h).
// kappa [ns][npts]; kq [nbands][nq][ns]; kavg [ns][nbands] or NULL.
static inline double ck_edge(double p0, double step, int h) {
    const double x = (double)h * step + p0;
    const double x2 = x * x;
    const double x4 = x2 * x2;
    const double x5 = x4 * x;
    return x5 * x5;
}

int orc_ck_from_lbl(const double *kappa, int ns, long long npts, double dwv, int nbands, const long long *first,
                    const int *count, const double *wv_left, const double *wv_right, int nq, const double *gq,
                    int n_pwrk, int nthreads, float *kq, double *kavg) {
    if (!kappa || ns < 1 || nbands < 1 || nq < 1 || n_pwrk < 2) return 1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 1)
    for (long long it = 0; it < (long long)ns * nbands; ++it) {
        const int b = (int)(it % nbands);
        const long long s_ = it / nbands;
        const double *kv = kappa + s_ * npts + first[b];
        const int n = count[b];
        double lo = kv[0], hi = kv[0];
        for (int h = 1; h < n; ++h) { lo = std::min(lo, kv[h]); hi = std::max(hi, kv[h]); }
        if (!(hi > lo)) {
            for (int r = 0; r < nq; ++r) kq[((long long)b * nq + r) * ns + s_] = (float)lo;
            if (kavg) kavg[s_ * nbands + b] = lo;
            continue;
        }
        const double p0 = std::pow(lo, 0.1), p1 = std::pow(hi, 0.1);
        const double step = (p1 - p0) / (double)(n_pwrk - 1);
        std::vector<long long> cnt((size_t)n_pwrk + 2, 0);
        for (int h = 1; h < n; ++h) {
            const double ki = (kv[h] + kv[h - 1]) / 2.0;
            int bin = std::max(0, (int)((std::pow(ki, 0.1) - p0) / step + 1.0));
            bin = std::min(bin, n_pwrk);
            cnt[(size_t)bin] += 1;
        }
        const double frac = dwv / (wv_right[b] - wv_left[b]);
        // suffix counts sfx[h] = sum_{bin = h .. n_pwrk-1} cnt, sfx[n_pwrk] = 0
        std::vector<long long> sfx((size_t)n_pwrk + 1, 0);
        for (int h = n_pwrk - 1; h >= 1; --h) sfx[(size_t)h] = sfx[(size_t)h + 1] + cnt[(size_t)h];
        auto g_at = [&](int h) { return 1.0 - (double)sfx[(size_t)h + 1] * frac; };
        auto k_at = [&](int h) { return 0.5 * (ck_edge(p0, step, h) + ck_edge(p0, step, h + 1)); };
        int t = 0;
        for (int r = 0; r < nq; ++r) {
            while (t < n_pwrk - 2 && !(g_at(t + 1) >= gq[r])) ++t;
            const double g0 = g_at(t), g1 = g_at(t + 1), k0 = k_at(t), k1 = k_at(t + 1);
            const double v = (g1 == g0) ? k1 : k0 + (k1 - k0) * (gq[r] - g0) / (g1 - g0);
            kq[((long long)b * nq + r) * ns + s_] = (float)v;
        }
        if (kavg) {
            double acc = 0.0;
            for (int h = 1; h < n_pwrk; ++h)
                if (cnt[(size_t)h]) acc += k_at(h) * ((double)cnt[(size_t)h] * frac);
            kavg[s_ * nbands + b] = acc;
        }
    }
    return 0;
}

int orc_packet_trace(const OrcPacketConfig *c, int f, int G, int p, int r, int max_steps, int32_t *rec, int *n,
                     uint32_t rng[4]) {
    if (!c || c->tile_a < 1 || 32 % c->tile_a || c->cpl < 0 || c->cpl > 4) return 1;
    if (c->cpl > 1 && c->mg_levels > 1) return 1;  // the multigrid march runs 32-cell packets
    double S[128], S2[128], st = 0;
    Packet<float>(*c).item(f, G, p, S, S2, &st, r, max_steps, rec, n, rng);
    return 0;
}

}  // extern "C"
