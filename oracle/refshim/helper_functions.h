/* Host stand-in for the CUDA-samples helper_functions.h (oracle pin build only). */
