// gi_model.h - the last step of the context model's score in the rescue's inference: the natural
// logarithm of a blended probability, in double precision, rounded to float. The reference takes
// the host C library's log of the same double (gpuinflate/rescue.cpp:1723-1733); the inferred
// values depend on these floats, so tests/test_gpu_model_log.py checks, over a large sample of the
// probabilities a model's counts give, that this function (CUDA's double log, accurate to within
// one unit in the last place) rounds to the same float as the host's log. Shared by gi_rescue.cu
// and that test's kernel.
#pragma once

__device__ __forceinline__ float model_log(double pr) { return __double2float_rn(log(pr)); }
