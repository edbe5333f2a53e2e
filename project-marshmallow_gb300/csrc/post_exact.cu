// post_exact.cu - the post chain in reproducible arithmetic (built with -fmad=false, mm_math.h
// pow): equal to the CPU restatement bit for bit.
#include "post_kernel.cuh"

namespace mm {

int launch_post_exact(const PostLaunch& p, int which, cudaStream_t s) { return post::launch<true>(p, which, s); }

}  // namespace mm
