// march_fast.cu - the cloud march in production arithmetic: FMA contraction, SFU exp2/log2 and
// rsqrt, texture-unit filtering.
#include "march_kernel.cuh"

namespace mm {

void prepare_march_fast() { march::prepare_march_kernels<false>(); }

int launch_march_fast(const MarchLaunch& p, int sampler, int format, int schedule, int half2, unsigned int* work,
                      int num_sms, cudaStream_t s) {
    (void)format;
    if (schedule == MM_SCHEDULE_TILED) {
        if (sampler == MM_SAMPLER_SOFTWARE) return march::launch_tiled<false, MM_SAMPLER_SOFTWARE>(p, s);
        // MM_MATH_FAST_HALF2 (FP16/BF16 density): full frames make their large-step decisions in half2
        return march::launch_tiled<false, MM_SAMPLER_HARDWARE>(p, s, half2 != 0);
    }
    if (sampler == MM_SAMPLER_SOFTWARE)
        return march::launch_persistent<false, MM_SAMPLER_SOFTWARE>(p, work, num_sms, s);
    return march::launch_persistent<false, MM_SAMPLER_HARDWARE>(p, work, num_sms, s);
}

}  // namespace mm
