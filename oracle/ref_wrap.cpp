// ref_wrap.cpp -- TEST INFRASTRUCTURE ONLY.  C entry points around the
// reference's own readT (code/read_tables.cpp) and interp3D
// (code/spline.cpp), compiled together with those files from the reference
// tree (see oracle/build.py).  The reference reads "../distr/tables/..."
// relative to the working directory; callers chdir accordingly.
#include <cstdio>
#include <cstring>
#include "param.h"
#include "definitions.h"
#include "functions.h"

myfloat prob[nT][nB], probg[nT][nB][nQ];  // defined by code/mc_gpu.cu:20 in the reference

extern "C" int ref_table_sizes(int *nt, int *nb, int *nq) { *nt = nT; *nb = nB; *nq = nQ; return grey; }

// Outputs: Tnb[nT], kP[nT], wvc[nB], kavg[nB], kq[nB][nT][nQ], prob[nT][nB],
// probg[nT][nB][nQ], kappamax at Tmax.
extern "C" int ref_readT(float Tmax, float *Tnb, float *kP, float *wvc, float *kavg, float *kq, float *prob_out,
                         float *probg_out, float *kappamax) {
    static NarrowBand nbands[nB];
    static myfloat prob_h[nB * nT], probg_h[nB * nT * nQ];
    memset(nbands, 0, sizeof nbands);
    readT(nbands, Tnb, kP, prob_h, probg_h, Tmax, kappamax);
    for (int b = 0; b < nB; ++b) {
        wvc[b] = nbands[b].wvc;
        kavg[b] = nbands[b].kavg;
        for (int t = 0; t < nT; ++t)
            for (int g = 0; g < nQ; ++g) kq[((size_t)b * nT + t) * nQ + g] = nbands[b].kq[t][g];
    }
    memcpy(prob_out, prob_h, sizeof prob_h);
    memcpy(probg_out, probg_h, sizeof probg_h);
    return 0;
}

// Spline-coarsened T on level `level` of grid_num levels (code/spline.cpp:35-116).
extern "C" int ref_interp3d(const float *Tfort, int level, float *Tout) {
    const int maxi_[] = {imax, imax / 2, imax / 4, imax / 8, imax / 16, imax / 32};
    const int maxj_[] = {jmax, jmax / 2, jmax / 4, jmax / 8, jmax / 16, jmax / 32};
    const int maxk_[] = {kmax, kmax / 2, kmax / 4, kmax / 8, kmax / 16, kmax / 32};
    Var_CPU v[grid_num];
    for (int g = 0; g < grid_num; ++g) v[g].mk_grid(maxi_[g], maxj_[g], maxk_[g], maxi_[0]);
    memcpy(v[0].T, Tfort, sizeof(float) * (imax + 2) * (jmax + 2) * (kmax + 2));
    interp3D(v);
    const size_t n = (size_t)(v[level].im + 2) * (v[level].jm + 2) * (v[level].km + 2);
    memcpy(Tout, v[level].T, n * sizeof(float));
    for (int g = 0; g < grid_num; ++g) v[g].destroyVar();
    return 0;
}
