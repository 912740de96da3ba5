// mc_march_pair.cu -- the two-cell march of the absorbing gas with black
// walls (mc_march_pair.cuh), instantiated apart from the general-medium
// variants (mc_march_gen.cu) so both compile in parallel.  Compiled with
// -fmad=false like the other march translation units.
#include "mc_march_pair.cuh"

namespace dnsmc {

int launch_march_pair(int mode, const MarchParams &p, int blocks, int threads, void *stream, bool trace, bool cv,
                      bool mom) {
    return launch_march_cells<false>(mode, p, blocks, threads, stream, trace, cv, mom);
}

int march_pair_occupancy(int mode, int threads, bool cv, bool mom, size_t smem) {
    return march_cells_occupancy<false>(mode, threads, cv, mom, smem);
}

int upload_sobol_dirs_pair(const uint32_t dirs[4][32]) {
    return (int)cudaMemcpyToSymbol(c_sobol, dirs, sizeof(uint32_t) * 4 * 32);
}

}  // namespace dnsmc
