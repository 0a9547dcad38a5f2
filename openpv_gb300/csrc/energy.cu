// energy.cu -- a11: FP64 energy-probe reductions on the device.
//
// CostFunctionSum<C>::calculateSumNoMask (probes/CostFunctionSum.hpp:86-108) sums a cost of
// every restricted neuron of one batch element in double.  Here one block owns one batch
// element: each thread accumulates a fixed strided subset in double, then a fixed-shape
// tree combines the partial sums, so repeated runs give identical bits (the order differs
// from the reference's sequential loop only by double rounding).
#include "pvgpu_internal.cuh"

namespace {

using pvgpu::Loc;

constexpr int kThreads = 512;

__device__ __forceinline__ double cost(int kind, double x, double tw, double maxCost, double qc) {
   if (kind == 0) return x * x;
   if (kind == 1) return fabs(x);
   double ax = fabs(x);
   return ax < tw ? ax * (1.0 - qc * ax) : maxCost;  // probes/CostFunctions.hpp:32-49
}

__global__ void __launch_bounds__(kThreads) cost_sum_kernel(Loc loc, const float *__restrict__ buf, int kind,
                                                            double tw, double maxCost, double qc,
                                                            double *__restrict__ out) {
   const int b = blockIdx.x;
   const float *bb = buf + (size_t)b * loc.numExt();
   const int64_t n = loc.numRes();
   double s = 0.0;
   for (int64_t k = threadIdx.x; k < n; k += kThreads) s += cost(kind, (double)bb[loc.kex(k)], tw, maxCost, qc);
   __shared__ double red[kThreads];
   red[threadIdx.x] = s;
   __syncthreads();
   for (int w = kThreads / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
   }
   if (threadIdx.x == 0) out[b] = red[0];
}

}  // namespace

extern "C" pvgpu_status pvgpu_cost_sum(const pvgpu_loc *loc, const float *bufExt, int kind, double p0, double p1,
                                       double *out, void *stream) {
   if (!loc || !pvgpu::loc_valid(*loc) || !bufExt || !out || kind < 0 || kind > 2) return PVGPU_ERR_BAD_ARG;
   if (loc->nbatch > 0x7fffffff) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   double tw = p0 + p1;
   cost_sum_kernel<<<loc->nbatch, kThreads, 0, pvgpu::as_stream(stream)>>>(pvgpu::to_loc(*loc), bufExt, kind, tw,
                                                                           0.5 * tw, 0.5 / tw, out);
   PVGPU_CHECK_LAUNCH("cost_sum");
   return PVGPU_OK;
}
