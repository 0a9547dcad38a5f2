// layer_update.cu -- a6..a9: GSyn accumulation, LCA membrane update and the ANN threshold.
//
// Element-wise and HBM-bound.  Every product and sum is rounded separately (__fmul_rn /
// __fadd_rn / __fdiv_rn), in the order the reference's C++ evaluates it, so the results
// equal the reference CPU path bit for bit (nvcc would otherwise contract a*b+c into an
// FMA).  The per-batch decay factor e = (float)exp(-dt/tau) is computed once per batch
// element per block in double, as HyPerLCAInternalStateBuffer.kpp:50 does per neuron.
#include "pvgpu_internal.cuh"

#include <cfloat>

namespace {

using pvgpu::Loc;

constexpr int kThreads = 256;
constexpr int kItems = 4;

struct Thresh {
   float VThresh, AMin, AMax, AShift, VWidth;
};

// HyPerActivityBuffer::updateBufferCPU then ANNActivityBuffer::applyVThresh / applyAMax
// (components/ANNActivityBuffer.cpp:490-558), on one neuron.
__device__ __forceinline__ float ann_threshold(float v, const Thresh &t) {
   float a = v;
   if (t.VThresh > -FLT_MAX) {
      float vtw = __fadd_rn(t.VThresh, t.VWidth);
      if (v < t.VThresh) {
         a = t.AMin;
      } else if (v < vtw) {
         float c = __fadd_rn(__fadd_rn(vtw, -t.AShift), -t.AMin);
         a = __fadd_rn(t.AMin, __fdiv_rn(__fmul_rn(c, __fadd_rn(v, -t.VThresh)), t.VWidth));
      } else {
         a = __fadd_rn(a, -t.AShift);
      }
   }
   if (t.AMax < FLT_MAX && a > t.AMax) a = t.AMax;
   return a;
}

// HyPerLCAInternalStateBuffer.kpp:52-61
__device__ __forceinline__ float lca_step(float v, float g, float a, float e, float si) {
   return __fadd_rn(__fmul_rn(e, v), __fmul_rn(__fadd_rn(1.0f, -e), __fadd_rn(g, __fmul_rn(si, a))));
}

// Decay factors of the (at most kMaxB) batch elements a block touches.
constexpr int kMaxB = 8;
__device__ __forceinline__ void block_decay(const double *dtAdapt, float tau, int64_t first, int64_t numNeurons,
                                            int nb, float *eS) {
   int bFirst = (int)(first / numNeurons);
   if (threadIdx.x < kMaxB) {
      int b = bFirst + threadIdx.x;
      eS[threadIdx.x] = b < nb ? (float)exp(-dtAdapt[b] / (double)tau) : 0.0f;
   }
}

__global__ void __launch_bounds__(kThreads) accumulate_kernel(int64_t n, int nch, float c0, float c1, float c2,
                                                              float c3, const float *__restrict__ gsyn,
                                                              float *__restrict__ g) {
   const float cs[4] = {c0, c1, c2, c3};
   for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
      float value = 0.0f;
      for (int ch = 0; ch < nch; ch++) value = __fadd_rn(value, __fmul_rn(cs[ch], gsyn[(size_t)ch * n + i]));
      g[i] = value;
   }
}

__global__ void __launch_bounds__(kThreads) lca_update_kernel(Loc loc, float si, const double *__restrict__ dtAdapt,
                                                              float tau, const float *__restrict__ g,
                                                              const float *__restrict__ aExt,
                                                              float *__restrict__ v) {
   const int64_t numNeurons = loc.numRes(), total = numNeurons * loc.nb;
   const int64_t first = (int64_t)blockIdx.x * kThreads * kItems;
   __shared__ float eS[kMaxB];
   block_decay(dtAdapt, tau, first, numNeurons, loc.nb, eS);
   __syncthreads();
   const int b0 = (int)(first / numNeurons);
#pragma unroll
   for (int it = 0; it < kItems; it++) {
      int64_t i = first + it * kThreads + threadIdx.x;
      if (i >= total) break;
      int b = (int)(i / numNeurons);
      int64_t k = i - (int64_t)b * numNeurons;
      float a = aExt[(size_t)b * loc.numExt() + loc.kex(k)];
      v[i] = lca_step(v[i], g[i], a, eS[b - b0], si);
   }
}

// MomentumLCAInternalStateBuffer.kpp:51-66, rounded as the reference's C++ evaluates it:
// drive = (1 - e)(G + si A); V = (e V + drive) + rate * prevDrive; prevDrive = drive.
__global__ void __launch_bounds__(kThreads) momentum_lca_kernel(Loc loc, float si, float rate,
                                                                const double *__restrict__ dtAdapt, float tau,
                                                                const float *__restrict__ g,
                                                                const float *__restrict__ aExt,
                                                                float *__restrict__ prevDrive, float *__restrict__ v) {
   const int64_t numNeurons = loc.numRes(), total = numNeurons * loc.nb;
   const int64_t first = (int64_t)blockIdx.x * kThreads * kItems;
   __shared__ float eS[kMaxB];
   block_decay(dtAdapt, tau, first, numNeurons, loc.nb, eS);
   __syncthreads();
   const int b0 = (int)(first / numNeurons);
#pragma unroll
   for (int it = 0; it < kItems; it++) {
      int64_t i = first + it * kThreads + threadIdx.x;
      if (i >= total) break;
      int b = (int)(i / numNeurons);
      int64_t k = i - (int64_t)b * numNeurons;
      const float e = eS[b - b0];
      const float a = aExt[(size_t)b * loc.numExt() + loc.kex(k)];
      const float drive = __fmul_rn(__fadd_rn(1.0f, -e), __fadd_rn(g[i], __fmul_rn(si, a)));
      v[i] = __fadd_rn(__fadd_rn(__fmul_rn(e, v[i]), drive), __fmul_rn(rate, prevDrive[i]));
      prevDrive[i] = drive;
   }
}

// ISTAInternalStateBuffer.kpp:46-60: V += ((float)dt / tau)(G - VThresh sign(A)).
__global__ void __launch_bounds__(kThreads) ista_kernel(Loc loc, float VThresh, const double *__restrict__ dtAdapt,
                                                        float tau, const float *__restrict__ g,
                                                        const float *__restrict__ aExt, float *__restrict__ v) {
   const int64_t numNeurons = loc.numRes(), total = numNeurons * loc.nb;
   for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
      int b = (int)(i / numNeurons);
      int64_t k = i - (int64_t)b * numNeurons;
      const float a = aExt[(size_t)b * loc.numExt() + loc.kex(k)];
      float sign = 0.0f;
      if (a != 0.0f) sign = __fdiv_rn(a, fabsf(a));
      const float q = __fdiv_rn((float)dtAdapt[b], tau);
      v[i] = __fadd_rn(v[i], __fmul_rn(q, __fadd_rn(g[i], -__fmul_rn(VThresh, sign))));
   }
}

__global__ void __launch_bounds__(kThreads) ann_kernel(Loc loc, Thresh t, const float *__restrict__ v,
                                                       float *__restrict__ aExt) {
   const int64_t numNeurons = loc.numRes(), total = numNeurons * loc.nb;
   for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
      int b = (int)(i / numNeurons);
      int64_t k = i - (int64_t)b * numNeurons;
      aExt[(size_t)b * loc.numExt() + loc.kex(k)] = ann_threshold(v[i], t);
   }
}

// The piecewise-linear transfer function given by vertices (ANNActivityBuffer::setVertices /
// applyVerticesANNActivityBufferOnGPU, components/ANNActivityBuffer.kpp:16-77): below the first
// vertex and from the last one on, the outer slopes; between vertices v and v + 1 the slope
// slopes[v + 1]; a potential equal to a vertex takes the vertex's activity, the last of equal
// vertices winning (jumps are continuous from the right).  Products and sums are rounded
// separately, as the CPU form of the same function.
__global__ void __launch_bounds__(kThreads) ann_vertices_kernel(Loc loc, int nv, const float *__restrict__ vV,
                                                                const float *__restrict__ vA,
                                                                const float *__restrict__ slopes,
                                                                const float *__restrict__ v, float *__restrict__ aExt) {
   const int64_t numNeurons = loc.numRes(), total = numNeurons * loc.nb;
   const int last = nv - 1;
   for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
      const int b = (int)(i / numNeurons);
      const int64_t k = i - (int64_t)b * numNeurons;
      const float x = v[i];
      float a = 0.0f;
      if (x < vV[0]) {
         a = __fadd_rn(vA[0], __fmul_rn(slopes[0], __fsub_rn(x, vV[0])));
      } else if (x >= vV[last]) {
         a = __fadd_rn(vA[last], __fmul_rn(slopes[nv], __fsub_rn(x, vV[last])));
      } else {
         for (int j = 0; j < last && x >= vV[j]; j++) {
            if (x == vV[j]) a = vA[j];
            else if (x < vV[j + 1]) a = __fadd_rn(vA[j], __fmul_rn(slopes[j + 1], __fsub_rn(x, vV[j])));
         }
      }
      aExt[(size_t)b * loc.numExt() + loc.kex(k)] = a;
   }
}

// GSynAccumulator -> HyPerLCAInternalStateBuffer -> ANNActivityBuffer in one pass.
__global__ void __launch_bounds__(kThreads) lca_layer_kernel(Loc loc, int nch, float c0, float c1, float c2, float c3,
                                                             float si, float tau, Thresh t,
                                                             const float *__restrict__ gsyn,
                                                             const double *__restrict__ dtAdapt,
                                                             float *__restrict__ v, float *__restrict__ aExt) {
   const int64_t numNeurons = loc.numRes(), total = numNeurons * loc.nb;
   const int64_t first = (int64_t)blockIdx.x * kThreads * kItems;
   const float cs[4] = {c0, c1, c2, c3};
   __shared__ float eS[kMaxB];
   block_decay(dtAdapt, tau, first, numNeurons, loc.nb, eS);
   __syncthreads();
   const int b0 = (int)(first / numNeurons);
#pragma unroll
   for (int it = 0; it < kItems; it++) {
      int64_t i = first + it * kThreads + threadIdx.x;
      if (i >= total) break;
      int b = (int)(i / numNeurons);
      int64_t k = i - (int64_t)b * numNeurons;
      float gv = 0.0f;
      for (int ch = 0; ch < nch; ch++) gv = __fadd_rn(gv, __fmul_rn(cs[ch], gsyn[(size_t)ch * total + i]));
      float *ap = aExt + (size_t)b * loc.numExt() + loc.kex(k);
      float vn = lca_step(v[i], gv, *ap, eS[b - b0], si);
      v[i] = vn;
      *ap = ann_threshold(vn, t);
   }
}

bool blocks_fit_batch(const Loc &loc) {
   // a block spans kThreads*kItems neurons: it must not touch more than kMaxB batch elements
   int64_t span = (int64_t)kThreads * kItems;
   return loc.numRes() * (kMaxB - 1) >= span;
}

}  // namespace

extern "C" pvgpu_status pvgpu_gsyn_accumulate(int64_t n, int numChannels, const float *coeffs, const float *gsyn,
                                              float *g, void *stream) {
   if (n <= 0 || numChannels < 0 || numChannels > 4 || (numChannels > 0 && (!coeffs || !gsyn)) || !g)
      return PVGPU_ERR_BAD_ARG;
   float c[4] = {0, 0, 0, 0};
   for (int i = 0; i < numChannels; i++) c[i] = coeffs[i];
   int64_t blocks = (n + kThreads - 1) / kThreads;
   if (blocks > 152 * 64) blocks = 152 * 64;
   accumulate_kernel<<<(unsigned)blocks, kThreads, 0, pvgpu::as_stream(stream)>>>(n, numChannels, c[0], c[1], c[2],
                                                                                  c[3], gsyn, g);
   PVGPU_CHECK_LAUNCH("gsyn_accumulate");
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_update(const pvgpu_loc *loc, int selfInteract, const double *dtAdapt, float tau,
                                         const float *g, const float *aExt, float *v, void *stream) {
   if (!loc || !pvgpu::loc_valid(*loc) || !dtAdapt || !g || !aExt || !v) return PVGPU_ERR_BAD_ARG;
   Loc l = pvgpu::to_loc(*loc);
   if (!blocks_fit_batch(l)) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   int64_t total = l.numRes() * l.nb;
   int64_t blocks = (total + kThreads * kItems - 1) / (kThreads * kItems);
   lca_update_kernel<<<(unsigned)blocks, kThreads, 0, pvgpu::as_stream(stream)>>>(l, selfInteract ? 1.0f : 0.0f,
                                                                                  dtAdapt, tau, g, aExt, v);
   PVGPU_CHECK_LAUNCH("lca_update");
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_momentum_lca_update(const pvgpu_loc *loc, int selfInteract, float momentumRate,
                                                  const double *dtAdapt, float tau, const float *g, const float *aExt,
                                                  float *prevDrive, float *v, void *stream) {
   if (!loc || !pvgpu::loc_valid(*loc) || !dtAdapt || !g || !aExt || !prevDrive || !v) return PVGPU_ERR_BAD_ARG;
   Loc l = pvgpu::to_loc(*loc);
   if (!blocks_fit_batch(l)) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   int64_t total = l.numRes() * l.nb;
   int64_t blocks = (total + kThreads * kItems - 1) / (kThreads * kItems);
   momentum_lca_kernel<<<(unsigned)blocks, kThreads, 0, pvgpu::as_stream(stream)>>>(
         l, selfInteract ? 1.0f : 0.0f, momentumRate, dtAdapt, tau, g, aExt, prevDrive, v);
   PVGPU_CHECK_LAUNCH("momentum_lca_update");
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_ista_update(const pvgpu_loc *loc, float VThresh, const double *dtAdapt, float tau,
                                          const float *g, const float *aExt, float *v, void *stream) {
   if (!loc || !pvgpu::loc_valid(*loc) || !dtAdapt || !g || !aExt || !v) return PVGPU_ERR_BAD_ARG;
   Loc l = pvgpu::to_loc(*loc);
   int64_t total = l.numRes() * l.nb;
   int64_t blocks = (total + kThreads - 1) / kThreads;
   if (blocks > 152 * 64) blocks = 152 * 64;
   ista_kernel<<<(unsigned)blocks, kThreads, 0, pvgpu::as_stream(stream)>>>(l, VThresh, dtAdapt, tau, g, aExt, v);
   PVGPU_CHECK_LAUNCH("ista_update");
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_ann_activity(const pvgpu_loc *loc, const float *v, float VThresh, float AMin, float AMax,
                                           float AShift, float VWidth, float *aExt, void *stream) {
   if (!loc || !pvgpu::loc_valid(*loc) || !v || !aExt) return PVGPU_ERR_BAD_ARG;
   if (VWidth < 0) {  // ANNActivityBuffer::setVertices reinterprets a negative width
      VThresh += VWidth;
      VWidth = -VWidth;
   }
   Loc l = pvgpu::to_loc(*loc);
   int64_t total = l.numRes() * l.nb;
   int64_t blocks = (total + kThreads - 1) / kThreads;
   if (blocks > 152 * 64) blocks = 152 * 64;
   ann_kernel<<<(unsigned)blocks, kThreads, 0, pvgpu::as_stream(stream)>>>(l, Thresh{VThresh, AMin, AMax, AShift, VWidth},
                                                                           v, aExt);
   PVGPU_CHECK_LAUNCH("ann_activity");
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_ann_vertices(const pvgpu_loc *loc, int numVertices, const float *verticesV,
                                           const float *verticesA, const float *slopes, const float *v, float *aExt,
                                           void *stream) {
   if (!loc || !pvgpu::loc_valid(*loc) || numVertices < 1 || !verticesV || !verticesA || !slopes || !v || !aExt)
      return PVGPU_ERR_BAD_ARG;
   Loc l = pvgpu::to_loc(*loc);
   int64_t total = l.numRes() * l.nb;
   int64_t blocks = (total + kThreads - 1) / kThreads;
   if (blocks > 152 * 64) blocks = 152 * 64;
   ann_vertices_kernel<<<(unsigned)blocks, kThreads, 0, pvgpu::as_stream(stream)>>>(l, numVertices, verticesV,
                                                                                    verticesA, slopes, v, aExt);
   PVGPU_CHECK_LAUNCH("ann_vertices");
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_lca_layer_update(const pvgpu_lca_layer_desc *d, const float *gsyn,
                                               const double *dtAdapt, float *v, float *aExt, void *stream) {
   if (!d || !pvgpu::loc_valid(d->loc) || !dtAdapt || !v || !aExt) return PVGPU_ERR_BAD_ARG;
   if (d->numChannels < 0 || d->numChannels > 4 || (d->numChannels > 0 && !gsyn)) return PVGPU_ERR_BAD_ARG;
   Loc l = pvgpu::to_loc(d->loc);
   if (!blocks_fit_batch(l)) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   float vt = d->VThresh, vw = d->VWidth;
   if (vw < 0) {
      vt += vw;
      vw = -vw;
   }
   int64_t total = l.numRes() * l.nb;
   int64_t blocks = (total + kThreads * kItems - 1) / (kThreads * kItems);
   lca_layer_kernel<<<(unsigned)blocks, kThreads, 0, pvgpu::as_stream(stream)>>>(
         l, d->numChannels, d->coeffs[0], d->coeffs[1], d->coeffs[2], d->coeffs[3], d->selfInteract ? 1.0f : 0.0f,
         d->tau, Thresh{vt, d->AMin, d->AMax, d->AShift, vw}, gsyn, dtAdapt, v, aExt);
   PVGPU_CHECK_LAUNCH("lca_layer_update");
   return PVGPU_OK;
}
