// ident.cu -- IdentDelivery (delivery/IdentDelivery.cpp:99-180) and the error layer's scaling
// (ErrScaleInternalStateBuffer::updateBufferCPU, components/ErrScaleInternalStateBuffer.cpp:41-53).
//
// IdentDelivery adds each presynaptic neuron's activity to the postsynaptic neuron at the same
// restricted position and feature: GSyn[b][k] += A_ext[b][kex(k)].  The dense form walks the
// restricted neurons; the sparse form walks the SparseList and skips entries in the halo, as the
// reference does.  Every GSyn element receives at most one contribution, so the result is the
// reference's bit for bit whatever the order.
#include "pvgpu_internal.cuh"

namespace {

using pvgpu::Loc;

constexpr int kThreads = 256;

__global__ void ident_dense_kernel(Loc pre, const float *__restrict__ aExt, float *__restrict__ gsyn) {
   const int64_t nRes = pre.numRes();
   const int b = blockIdx.y;
   const float *ab = aExt + (size_t)b * pre.numExt();
   float *gb = gsyn + (size_t)b * nRes;
   for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nRes; k += (int64_t)gridDim.x * blockDim.x)
      gb[k] += ab[pre.kex(k)];
}

__global__ void ident_sparse_kernel(Loc pre, const pvgpu_entry *__restrict__ entries,
                                    const int64_t *__restrict__ numActive, float *__restrict__ gsyn) {
   const int b = blockIdx.y;
   const int64_t n = numActive[b];
   const pvgpu_entry *eb = entries + (size_t)b * pre.numExt();
   float *gb = gsyn + (size_t)b * pre.numRes();
   const int nxExt = pre.nxExt(), nyExt = pre.nyExt();
   for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
      const pvgpu_entry e = eb[i];
      const int f = (int)(e.index % pre.nf);
      const int xe = (int)((e.index / pre.nf) % nxExt);
      const int ye = (int)(e.index / ((uint32_t)pre.nf * nxExt));
      const int x = xe - pre.lt, y = ye - pre.up;
      if (x < 0 || x >= pre.nx || y < 0 || y >= pre.ny || ye >= nyExt) continue;
      gb[((size_t)y * pre.nx + x) * pre.nf + f] += e.value;
   }
}

__global__ void scale_kernel(int64_t n, float s, float *__restrict__ v) {
   for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
      v[k] *= s;
}

}  // namespace

extern "C" pvgpu_status pvgpu_deliver_ident(const pvgpu_loc *pre, const pvgpu_loc *post, const pvgpu_entry *entries,
                                            const int64_t *numActive, const float *aExt, float *gsyn, void *stream) {
   if (!pre || !post || !gsyn || !pvgpu::loc_valid(*pre) || !pvgpu::loc_valid(*post)) return PVGPU_ERR_BAD_ARG;
   if (entries ? !numActive : !aExt) return PVGPU_ERR_BAD_ARG;
   if (pre->nbatch != post->nbatch || pre->nx != post->nx || pre->ny != post->ny || pre->nf != post->nf)
      return PVGPU_ERR_ILLEGAL_GEOMETRY;  // IdentConn requires the same restricted sizes
   const Loc l = pvgpu::to_loc(*pre);
   if (l.numExt() > 0xffffffffLL || pre->nbatch > 65535) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   cudaStream_t s = pvgpu::as_stream(stream);
   const int64_t work = entries ? l.numExt() : l.numRes();
   int64_t blocks = (work + kThreads - 1) / kThreads;
   if (blocks > 152 * 8) blocks = 152 * 8;
   dim3 grid((unsigned)(blocks > 0 ? blocks : 1), pre->nbatch);
   if (entries) ident_sparse_kernel<<<grid, kThreads, 0, s>>>(l, entries, numActive, gsyn);
   else ident_dense_kernel<<<grid, kThreads, 0, s>>>(l, aExt, gsyn);
   PVGPU_CHECK_LAUNCH("deliver_ident");
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_err_scale(int64_t n, float errScale, float *v, void *stream) {
   if (n < 0 || (n > 0 && !v)) return PVGPU_ERR_BAD_ARG;
   if (n == 0) return PVGPU_OK;
   int64_t blocks = (n + kThreads - 1) / kThreads;
   if (blocks > 152 * 8) blocks = 152 * 8;
   scale_kernel<<<(unsigned)blocks, kThreads, 0, pvgpu::as_stream(stream)>>>(n, errScale, v);
   PVGPU_CHECK_LAUNCH("err_scale");
   return PVGPU_OK;
}
