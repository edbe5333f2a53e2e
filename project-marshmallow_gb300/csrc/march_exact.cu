// march_exact.cu - the cloud march in reproducible arithmetic.  Built with -fmad=false: no
// contraction into FMA, IEEE division and square root, mm_math.h elementary functions.  With the
// software sampler its output equals the FP32 CPU oracle bit for bit.
#include "march_kernel.cuh"

namespace mm {

void prepare_march_exact() { march::prepare_march_kernels<true>(); }

int launch_march_exact(const MarchLaunch& p, int sampler, int schedule, unsigned int* work, int num_sms,
                       cudaStream_t s) {
    if (schedule == MM_SCHEDULE_TILED) {
        if (sampler == MM_SAMPLER_SOFTWARE) return march::launch_tiled<true, MM_SAMPLER_SOFTWARE>(p, s);
        return march::launch_tiled<true, MM_SAMPLER_HARDWARE>(p, s);
    }
    if (sampler == MM_SAMPLER_SOFTWARE)
        return march::launch_persistent<true, MM_SAMPLER_SOFTWARE>(p, work, num_sms, s);
    return march::launch_persistent<true, MM_SAMPLER_HARDWARE>(p, work, num_sms, s);
}

}  // namespace mm
