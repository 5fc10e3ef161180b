// Exclusion correction of the Ewald sum and exception pairs as standalone
// kernels, one thread per pair (the step itself runs them fused into the
// per-term kernel of k_bonded.cu; these serve the per-phase profile).
// The per-pair arithmetic is in nxm_pairterms.cuh.
#include "nxm_pairterms.cuh"

namespace nxm {

template <bool MIXED>
__global__ void __launch_bounds__(256) k_exclusions(DevView v, int energy) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    TermE<MIXED> e = 0;
    int sys = 0;
    if (t < v.nex) e = exclusion_pair<MIXED>(v, t, sys);
    if (energy) energy_add_t(v.E, sys, E_EXCL, e);
}

template <bool MIXED>
__global__ void __launch_bounds__(256) k_exceptions(DevView v, int energy) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    TermE<MIXED> e = 0;
    int sys = 0;
    if (t < v.nxc) e = exception_pair<MIXED>(v, t, sys);
    if (energy) energy_add_t(v.E, sys, E_EXCEPT, e);
}
void launch_exceptions(const DevView &v, int energy, cudaStream_t st) {
    if (v.nxc == 0) return;
    int nb = (v.nxc + 255) / 256;
    if (v.mixed)
        k_exceptions<true><<<nb, 256, 0, st>>>(v, energy);
    else
        k_exceptions<false><<<nb, 256, 0, st>>>(v, energy);
}

void launch_exclusions(const DevView &v, int energy, cudaStream_t st) {
    if (v.nex == 0) return;
    int nb = (v.nex + 255) / 256;
    if (v.mixed)
        k_exclusions<true><<<nb, 256, 0, st>>>(v, energy);
    else
        k_exclusions<false><<<nb, 256, 0, st>>>(v, energy);
}

}  // namespace nxm
