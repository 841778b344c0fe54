// cuew (the CUDA loader the reference uses) declares the CUDA driver and NVRTC
// API; for the compile check the toolkit's own headers declare them.
#include <cuda.h>
#include <nvrtc.h>
