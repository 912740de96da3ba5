// mc_march_gen.cu -- the march kernel for the general medium (particles with
// Henyey-Greenstein scattering, grey diffuse walls), instantiated apart from
// the absorbing-gas variants so both compile in parallel.
#include "mc_march.cuh"

namespace dnsmc {

int launch_march_gen(int mode, const MarchParams &p, int blocks, int threads, void *stream, bool trace, bool cv,
                     bool mom) {
    return launch_march_variant<true>(mode, p, blocks, threads, (cudaStream_t)stream, trace, cv, mom);
}

int march_gen_occupancy(int mode, int threads, bool cv, bool mom, size_t smem) {
    return march_variant_occupancy<true>(mode, threads, cv, mom, smem);
}

int upload_sobol_dirs_gen(const uint32_t dirs[4][32]) {
    return (int)cudaMemcpyToSymbol(c_sobol, dirs, sizeof(uint32_t) * 4 * 32);
}

}  // namespace dnsmc
