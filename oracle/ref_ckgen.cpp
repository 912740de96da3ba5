// ref_ckgen.cpp -- TEST INFRASTRUCTURE ONLY.  A C entry point around the
// reference's own k-distribution routine, correlatedKT
// (distr/correlatedK.cpp:145-300), compiled from the reference sources where
// they lie (oracle/build.py) so the tests can check the oracle's restatement
// (orc_ck_from_lbl) against it.  The reference fixes nT (52), nQuad (16, with
// its gq points) and n_pwrk (10000) at compile time in distr/classes.h; the
// routine writes per-temperature error files into errors/ of the working
// directory, so the call runs with the caller's directory current.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sys/stat.h>
#include <unistd.h>

#include "classes.h"
#include "functions.h"

extern "C" {

int ref_ck_sizes(int *nt, int *nq, int *npwrk) {
    *nt = nT;
    *nq = nQuad;
    *npwrk = n_pwrk;
    return 0;
}

void ref_ck_gq(double *out) {
    for (int r = 0; r < nQuad; ++r) out[r] = gq[r];
}

// kappa [nT][npts], wvn [npts]; band b = points [first[b], first[b] + count[b]).
// kq out [nT][nbands][nQuad].
int ref_ck_correlatedKT(const double *kappa, long long npts, const double *wvn, int nbands, const long long *first,
                        const int *count, const double *wv_left, const double *wv_right, const char *workdir,
                        double *kq) {
    char old[4096];
    if (!getcwd(old, sizeof old)) return 1;
    if (chdir(workdir) != 0) return 2;
    mkdir("errors", 0755);
    TempBand *tb = new TempBand[nT];
    for (int i = 0; i < nT; ++i) {
        tb[i].T = Tinit + DT * i;
        tb[i].allocNarrBands(nbands);
        tb[i].totbands = nbands;
        for (int j = 0; j < nbands; ++j) {
            NarrowBand2 &nb = tb[i].narrband[j];
            nb.allocVar(count[j]);
            nb.size = count[j];
            nb.wv_left = wv_left[j];
            nb.wv_right = wv_right[j];
            nb.wvc = 0.5 * (wv_left[j] + wv_right[j]);
            for (int h = 0; h < count[j]; ++h) {
                nb.wvn[h] = wvn[first[j] + h];
                nb.kvn[h] = kappa[(long long)i * npts + first[j] + h];
            }
        }
    }
    correlatedKT(tb);
    for (int i = 0; i < nT; ++i)
        for (int j = 0; j < nbands; ++j)
            for (int r = 0; r < nQuad; ++r) kq[((long long)i * nbands + j) * nQuad + r] = tb[i].narrband[j].kq[r];
    for (int i = 0; i < nT; ++i) {
        for (int j = 0; j < nbands; ++j) {
            NarrowBand2 &nb = tb[i].narrband[j];
            delete[] nb.wvn; delete[] nb.kvn; delete[] nb.prob_lbl; delete[] nb.cuprob_lbl;
        }
        delete[] tb[i].narrband;
    }
    delete[] tb;
    return chdir(old) == 0 ? 0 : 3;
}

}  // extern "C"
