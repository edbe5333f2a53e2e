// shadow_exact.cu - the mesh cloud-shadow march in reproducible arithmetic (built with
// -fmad=false, mm_math.h elementary functions).  With the software sampler its output equals
// the FP32 CPU restatement bit for bit.
#include "shadow_kernel.cuh"

namespace mm {

int launch_shadow_exact(const ShadowLaunch& p, int sampler, cudaStream_t s) {
    if (sampler == MM_SAMPLER_SOFTWARE) return shadow::launch<true, MM_SAMPLER_SOFTWARE>(p, s);
    return shadow::launch<true, MM_SAMPLER_HARDWARE>(p, s);
}

}  // namespace mm
