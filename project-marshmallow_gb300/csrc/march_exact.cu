// march_exact.cu - the cloud march in reproducible arithmetic.  Built with -fmad=false: no
// contraction into FMA, IEEE division and square root, mm_math.h elementary functions.  With the
// software sampler its output equals the FP32 CPU oracle bit for bit.  This unit holds the
// texture-unit sampler's kernels; march_exact_sw.cu the software sampler's (two units compile in
// parallel).
#include "march_kernel.cuh"

namespace mm {

void prepare_march_exact() {
    march::pool_carveout<true, MM_SAMPLER_HARDWARE, false>();
    march::pool_carveout<true, MM_SAMPLER_HARDWARE, true>();
    prepare_march_exact_sw();
}

int launch_march_exact(const MarchLaunch& p, int sampler, int schedule, unsigned int* work, int num_sms,
                       cudaStream_t s) {
    if (sampler == MM_SAMPLER_SOFTWARE) return launch_march_exact_sw(p, schedule, work, num_sms, s);
    if (schedule == MM_SCHEDULE_TILED) return march::launch_tiled<true, MM_SAMPLER_HARDWARE>(p, s);
    return march::launch_persistent<true, MM_SAMPLER_HARDWARE>(p, work, num_sms, s);
}

}  // namespace mm
