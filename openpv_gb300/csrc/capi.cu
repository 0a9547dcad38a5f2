// capi.cu -- library-level entry points: version, status strings, last-error record.
#include "pvgpu_internal.cuh"

#include <cstdio>
#include <cstring>

namespace pvgpu {

static thread_local char g_last_error[256] = "";

pvgpu_status record_cuda_error(cudaError_t err, const char *where) {
   std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s", where, cudaGetErrorString(err));
   if (err == cudaErrorMemoryAllocation) return PVGPU_ERR_OOM;
   return PVGPU_ERR_LAUNCH;
}

pvgpu_status record_message(pvgpu_status status, const char *message) {
   std::snprintf(g_last_error, sizeof(g_last_error), "%s", message);
   return status;
}

}  // namespace pvgpu

extern "C" const char *pvgpu_version(void) { return "pvgpu 0.1 (sm_103a)"; }

extern "C" const char *pvgpu_status_string(pvgpu_status s) {
   switch (s) {
      case PVGPU_OK: return "ok";
      case PVGPU_ERR_BAD_ARG: return "bad argument";
      case PVGPU_ERR_OOM: return "out of device memory";
      case PVGPU_ERR_LAUNCH: return "kernel launch or CUDA runtime error";
      case PVGPU_ERR_TIMEOUT: return "bounded device wait timed out";
      case PVGPU_ERR_UNSUPPORTED_SHAPE: return "shape not supported by this library";
      case PVGPU_ERR_ILLEGAL_GEOMETRY: return "geometry rejected by OpenPV's patch rules";
   }
   return "unknown status";
}

extern "C" const char *pvgpu_last_error(void) { return pvgpu::g_last_error; }
