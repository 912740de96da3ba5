// mc_march_gen.cu -- the march of the general medium (particles with
// Henyey-Greenstein scattering, grey diffuse walls): the two-cell march of
// mc_march_pair.cuh with GEN, instantiated apart from the absorbing-gas
// variants so both compile in parallel.
#include "mc_march_pair.cuh"

namespace dnsmc {

int launch_march_gen(int mode, const MarchParams &p, int blocks, int threads, void *stream, bool trace, bool cv,
                     bool mom) {
    return launch_march_cells<true>(mode, p, blocks, threads, stream, trace, cv, mom);
}

int march_gen_occupancy(int mode, int threads, bool cv, bool mom, size_t smem) {
    return march_cells_occupancy<true>(mode, threads, cv, mom, smem);
}

int upload_sobol_dirs_gen(const uint32_t dirs[4][32]) {
    return (int)cudaMemcpyToSymbol(c_sobol, dirs, sizeof(uint32_t) * 4 * 32);
}

}  // namespace dnsmc
