/* Host stand-in for the CUDA-samples helper_string.h (oracle pin build only). */
