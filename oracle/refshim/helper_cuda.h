/* Host stand-in for the CUDA-samples helper_cuda.h (oracle pin build only). */
#ifndef XD_REFSHIM_HELPER_CUDA_H
#define XD_REFSHIM_HELPER_CUDA_H
#define checkCudaErrors(x) (x)
#endif
