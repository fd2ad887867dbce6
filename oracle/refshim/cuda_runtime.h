/* Host stand-in for <cuda_runtime.h> (oracle pin build only). */
#ifndef XD_REFSHIM_CUDA_RUNTIME_H
#define XD_REFSHIM_CUDA_RUNTIME_H
#include "vector_types.h"
#endif
