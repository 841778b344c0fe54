// The OptiX names the LuxCore CUDA headers mention (declarations only, for
// the compile check of the LuxRays binding).
typedef int OptixResult;
#define OPTIX_SUCCESS 0
inline const char *optixGetErrorName(OptixResult) { return ""; }
inline const char *optixGetErrorString(OptixResult) { return ""; }
typedef struct OptixDeviceContext_t *OptixDeviceContext;
