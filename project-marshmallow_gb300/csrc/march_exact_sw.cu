// march_exact_sw.cu - the exact-arithmetic march with the software trilinear sampler (see
// march_exact.cu; built with -fmad=false).  Its output equals the FP32 CPU oracle bit for bit.
#include "march_kernel.cuh"

namespace mm {

void prepare_march_exact_sw() {
    march::pool_carveout<true, MM_SAMPLER_SOFTWARE, false>();
    march::pool_carveout<true, MM_SAMPLER_SOFTWARE, true>();
}

int launch_march_exact_sw(const MarchLaunch& p, int schedule, unsigned int* work, int num_sms, cudaStream_t s) {
    if (schedule == MM_SCHEDULE_TILED) return march::launch_tiled<true, MM_SAMPLER_SOFTWARE>(p, s);
    return march::launch_persistent<true, MM_SAMPLER_SOFTWARE>(p, work, num_sms, s);
}

}  // namespace mm
