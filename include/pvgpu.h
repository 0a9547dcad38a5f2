/*
 * pvgpu.h -- C ABI of the GB300-native (sm_103a) synaptic-delivery + LCA-update path.
 *
 * One shared library, libpvgpu.so, built from openpv_gb300/csrc.  Every entry point:
 *   - takes device pointers in the OpenPV layouts (activity [nbatch][nyExt][nxExt][nf],
 *     GSyn channel [nbatch][ny][nx][nf], shared weights [kernel][nyp][nxp][nfp], all FP32
 *     unless stated),
 *   - takes an explicit CUDA stream (a cudaStream_t passed as void*; NULL = legacy default
 *     stream) and never synchronises it, so a sequence of calls can be captured in a CUDA
 *     graph,
 *   - returns a pvgpu_status and never aborts.  The reference's handleError
 *     (arch/cuda/cuda_util.hpp:14-27) turns every CUDA error into Fatal(); adapters that
 *     want that behaviour test the status and call their own Fatal.
 *
 * Each declaration names the reference interface it replaces (paths relative to the
 * OpenPV source tree).
 */
#ifndef PVGPU_H_
#define PVGPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
   PVGPU_OK = 0,
   PVGPU_ERR_BAD_ARG = 1,           /* null pointer, negative size, inconsistent locs */
   PVGPU_ERR_OOM = 2,               /* device allocation failed */
   PVGPU_ERR_LAUNCH = 3,            /* kernel launch or CUDA runtime error */
   PVGPU_ERR_TIMEOUT = 4,           /* a bounded device-side wait gave up */
   PVGPU_ERR_UNSUPPORTED_SHAPE = 5, /* legal OpenPV geometry the library does not handle */
   PVGPU_ERR_ILLEGAL_GEOMETRY = 6   /* geometry OpenPV itself rejects (PatchGeometry::verifyPatchSize) */
} pvgpu_status;

/* PVHalo / PVLayerLoc (include/PVLayerLoc.h:14-26), batch-local fields. */
typedef struct {
   int lt, rt, dn, up;
} pvgpu_halo;

typedef struct {
   int nbatch, nx, ny, nf;
   pvgpu_halo halo;
} pvgpu_loc;

/* SparseList<float>::Entry (structures/SparseList.hpp:19-22): extended index + value. */
typedef struct {
   uint32_t index;
   float value;
} pvgpu_entry;

/* Connection geometry shared by the delivery calls: the presynaptic (source) layer,
 * the postsynaptic (target) layer and the presynaptic patch size nxp x nyp (nfp is
 * post.nf).  Mirrors the geometry fields of recv_pre_params / recv_post_params
 * (cudakernels/CudaRecvPre.hpp:19-45, cudakernels/CudaRecvPost.hpp:18-80). */
typedef struct {
   pvgpu_loc pre;
   pvgpu_loc post;
   int nxp, nyp;
   float dt_factor; /* 1 for convolve delivery (HyPerDelivery.cpp:26-81) */
} pvgpu_conn_desc;

/* Delivery numerics. */
enum {
   PVGPU_DELIVER_FAST = 0,           /* FP32 with fused multiply-add, tiled order */
   PVGPU_DELIVER_REFERENCE_ORDER = 1 /* FP32, separately rounded products and sums in the
                                        reference's single-thread order: bit-identical to the
                                        reference CPU path run with -t 1 */
};

/* ---- library ------------------------------------------------------------ */
const char *pvgpu_version(void);
const char *pvgpu_status_string(pvgpu_status s);
/* Last CUDA error string recorded by a failing call on this thread. */
const char *pvgpu_last_error(void);

/* Diagnostic, no counterpart in the reference (whose CUDA errors are fatal): runs one CTA whose
 * warp waits on an mbarrier that nothing arrives at, bounded by limitNs (0 < limitNs <= 1 s) of
 * the device's global timer, and takes the path every kernel here takes when a bounded wait
 * expires (abort flag seen by the other roles, tensor memory freed, status reported).
 * Synchronous; hostOut2 receives {1 if the wait expired, nanoseconds waited}; returns
 * PVGPU_ERR_TIMEOUT when the wait expired (the expected result) and leaves the context usable. */
pvgpu_status pvgpu_selftest_wait_expiry(uint64_t limitNs, long long *hostOut2, void *stream);

/* ---- a1: active-index compaction ------------------------------------------------------
 * Replaces DataStore::updateActiveIndices (columns/DataStore.cpp:46-66), which the reference
 * runs on the host after a device->host copy.  Stable: entries of each batch element are in
 * ascending extended index, value = the exact activity float; numActive[b] (long in the
 * reference) receives the count.  entries has capacity numExt per batch element.
 * One pass over the activity (chunks of 16384 values; a decoupled look-back carries the chunk
 * prefixes).  Scratch: `scratch` (device, 8-byte aligned, >= pvgpu_compact_scratch_bytes) holds
 * a ticket word and one status word per chunk; the call clears it on the stream first.
 * entries must be 8-byte aligned.  numActive[b] = -1 reports a look-back that gave up waiting
 * (bounded device wait; never expected). */
size_t pvgpu_compact_scratch_bytes(int nbatch, int64_t numExt);
pvgpu_status pvgpu_compact_active(
      const float *aExt,
      int nbatch,
      int64_t numExt,
      pvgpu_entry *entries,
      int64_t *numActive,
      void *scratch,
      size_t scratchBytes,
      void *stream);

/* The same compaction with no device allocation and no caller scratch.  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory at the call site -- loops
 * that must not incur the implicit device synchronisation cudaMalloc / cudaFree may cause, and
 * hosts whose device memory all belongs to their own pool allocator.  The ticket and chunk
 * statuses live in a fixed 1 MiB array inside the library's device image (loaded once per
 * device, kept until the process exits), which limits a call to
 * nbatch * ceil(numExt / 16384) <= 131071; larger calls return PVGPU_ERR_BAD_ARG with a message
 * in pvgpu_last_error().  Each call clears the part of the array it uses (cudaMemsetAsync on the
 * stream) before its kernel reads it.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress, with that device current) and caches it per device ordinal for
 * the life of the process (not across cudaDeviceReset); make that first call before any stream
 * capture.  All calls share the one array: calls that overlap on the GPU (concurrent streams,
 * or several host threads) race on it and must be serialised by the caller.  Output equals
 * pvgpu_compact_active's. */
pvgpu_status pvgpu_compact_active_noalloc(
      const float *aExt,
      int nbatch,
      int64_t numExt,
      pvgpu_entry *entries,
      int64_t *numActive,
      void *stream);

/* ---- a4: presynaptic-perspective delivery -----------------------------------------------
 * Replaces CudaRecvPre::do_run / HyPerLayer_recv_pre (cudakernels/CudaRecvPre.cu:10-101)
 * driven by PresynapticPerspectiveGPUDelivery::deliver (delivery/PresynapticPerspectiveGPUDelivery.cpp:198-270),
 * with the CPU semantics of PresynapticPerspectiveConvolveDelivery::deliver
 * (delivery/PresynapticPerspectiveConvolveDelivery.cpp:61-192).  Shared weights, one arbor.
 * Sparse input: entries/numActive (SparseList per batch element, stride numPreExt); pass
 * entries = NULL to read the dense activity aExt instead (zeros skipped).  GSyn of the
 * channel ([nbatch][post restricted]) is accumulated into.  No atomics: each GSyn element
 * is owned by one thread and receives its contributions in the reference's order
 * (patch row, then ascending presynaptic index). */
pvgpu_status pvgpu_deliver_pre(
      const pvgpu_conn_desc *conn,
      const pvgpu_entry *entries,
      const int64_t *numActive,
      const float *aExt,
      const float *weights,
      float *gsyn,
      int mode,
      void *stream);

/* ---- a5: postsynaptic-perspective delivery ----------------------------------------------
 * Replaces CudaRecvPost::do_run (cudnnConvolutionForward plus the NHWC<->NCHW permutes,
 * cudakernels/CudaRecvPost.cpp:357-389, arch/cuda/CudaKernel.cu:20-135) driven by
 * PostsynapticPerspectiveGPUDelivery::deliver (delivery/PostsynapticPerspectiveGPUDelivery.cpp:239-281),
 * with the semantics of PostsynapticPerspectiveConvolveDelivery::deliver
 * (delivery/PostsynapticPerspectiveConvolveDelivery.cpp:56-151).
 * conn describes the connection pre->post; postWeights are the post-perspective weights
 * (kernels of the post->pre geometry, patch nxpPost x nypPost x pre.nf, as produced by
 * TransposeWeights::transposeShared, or the original connection's weights for a
 * TransposeConn).  Reads the whole unshrunken receptive field from the extended
 * presynaptic activity, which needs pre.halo >= the connection's margin. */
pvgpu_status pvgpu_deliver_post(
      const pvgpu_conn_desc *conn,
      const float *aExt,
      const float *postWeights,
      float *gsyn,
      int mode,
      void *stream);

/* ---- LIF layer update ----------------------------------------------------------------------
 * LIFActivityComponent::updateActivity (components/LIFActivityComponent.cpp:332-942; CPU-only in
 * the reference) on the device, one step for every restricted neuron: noise on the EXC, INH and
 * INHB GSyn channels (gsynHead holds the three, each nbatch * nx*ny*nf), the conductance and
 * membrane update of `method` ('a' arma, the reference default; 'b' Heun; 'o' exponential Euler),
 * the threshold relaxation and the spike (A = 1 at the extended index, V = Vrest,
 * Vth += deltaVth, G_IB += deltaGIB).  rnd, V, Vth, GE, GI, GIB are restricted and updated in
 * place; aExt's halo is not written.  'b' equals the reference bit for bit; 'a' and 'o' differ
 * only by the device's expf / powf / logf in their per-neuron filter coefficients. */
typedef struct {
   uint32_t s0, s1, s2, s3; /* taus_uint4 (include/pv_types.h:54-59): last output, generator words */
} pvgpu_taus;

typedef struct { /* LIFParams (components/LIFActivityComponent.hpp:22-45), same fields and order */
   float Vrest, Vexc, Vinh, VinhB;
   float VthRest, tau, tauVth, deltaVth, deltaGIB;
   float noiseAmpE, noiseAmpI, noiseAmpIB, noiseFreqE, noiseFreqI, noiseFreqIB;
   float tauE, tauI, tauIB;
} pvgpu_lif_params;

pvgpu_status pvgpu_lif_update(
      const pvgpu_loc *loc,
      char method,
      const pvgpu_lif_params *params,
      float dt,
      pvgpu_taus *rnd,
      float *V,
      float *Vth,
      float *GE,
      float *GI,
      float *GIB,
      const float *gsynHead,
      float *aExt,
      void *stream);

/* cl_random_init (utils/cl_random.c) on the device: element i seeded with i + seed. */
pvgpu_status pvgpu_taus_init(pvgpu_taus *state, int64_t count, uint32_t seed, void *stream);

/* ---- .pvp activity frames, built on the device -------------------------------------------
 * Sparse frame payloads for PVP_ACT_SPARSEVALUES_FILE_TYPE files: each batch element's SparseList
 * (extended indices, stride numExt) as the file stores it -- halo entries dropped, indices made
 * restricted, order kept (SparseLayerBatchGatherScatter::gather then SparseList::crop,
 * io/SparseLayerBatchGatherScatter.cpp:24-80, structures/SparseList.hpp:76-110).  out has
 * capacity nx*ny*nf entries per batch element (stride nx*ny*nf); counts[b] receives the number
 * kept. */
pvgpu_status pvgpu_pvp_sparse_frames(
      const pvgpu_loc *loc,
      const pvgpu_entry *entries,
      const int64_t *numActive,
      pvgpu_entry *out,
      int32_t *counts,
      void *stream);
/* Dense frame payloads (PVP_NONSPIKING_ACT_FILE_TYPE): the restricted activity of each batch
 * element, [nbatch][ny][nx][nf]. */
pvgpu_status pvgpu_pvp_dense_frames(const pvgpu_loc *loc, const float *aExt, float *out, void *stream);
/* A file's sparse frames (restricted entries, stride nx*ny*nf, counts[b]) into the extended
 * activity, which is zeroed first; an index outside the layer sets *badIndex (device int) to 1
 * and is skipped. */
pvgpu_status pvgpu_pvp_scatter_sparse(
      const pvgpu_loc *loc,
      const pvgpu_entry *fileEntries,
      const int32_t *counts,
      float *aExt,
      int32_t *badIndex,
      void *stream);

/* ---- a4 / a5 on the tensor cores ---------------------------------------------------------
 * The same deliveries for a one-to-one connection (pre and post of equal nx, ny; pre.nf and
 * post.nf multiples of 32; nxp <= 9; equal halo on all sides, at least the connection's
 * margin), computed as an implicit GEMM on the tcgen05 tensor cores with each FP32 operand
 * split into two TF32 parts and three TF32 products per term, accumulated in short tensor-core
 * chains that are summed in FP32 with round-to-nearest: the FAST mode's accuracy class.  Reads the dense
 * extended presynaptic activity (the layer's activity buffer, which the reference's GPU
 * deliveries also receive: recv_pre_params.preData, cudakernels/CudaRecvPre.hpp:19-45), so the
 * cost does not depend on the activity's density.  GSyn of the channel is accumulated into.
 * pvgpu_deliver_tc_workspace_bytes is 0 for a connection these entries do not take.
 * `workspace` (device, 16-byte aligned, >= pvgpu_deliver_tc_workspace_bytes) holds the split
 * (and, for the presynaptic entry, transposed) weights; calls that overlap on the GPU need
 * separate workspaces.  Other shapes return PVGPU_ERR_UNSUPPORTED_SHAPE: use
 * pvgpu_deliver_pre / pvgpu_deliver_post.  No reference counterpart as an entry point; it
 * replaces the same calls as those two. */
size_t pvgpu_deliver_tc_workspace_bytes(const pvgpu_conn_desc *conn);
pvgpu_status pvgpu_deliver_post_tc(
      const pvgpu_conn_desc *conn,
      const float *aExt,
      const float *postWeights,
      float *gsyn,
      void *workspace,
      size_t workspaceBytes,
      void *stream);
pvgpu_status pvgpu_deliver_pre_tc(
      const pvgpu_conn_desc *conn,
      const float *aExt,
      const float *weights,
      float *gsyn,
      void *workspace,
      size_t workspaceBytes,
      void *stream);
/* 1 if a bounded device-side wait of a tensor-core delivery gave up since the last call (and
 * clears the flag); synchronises the device. */
int pvgpu_deliver_tc_check_error(void);

/* Post weights from pre weights: TransposeWeights::transposeShared (utils/TransposeWeights.cpp:56-115)
 * on the device, for WeightsPair::finalizeUpdate (components/WeightsPair.cpp:261-277). */
pvgpu_status pvgpu_transpose_weights(const pvgpu_conn_desc *conn, const float *preWeights, float *postWeights, void *stream);

/* IdentDelivery::deliver (delivery/IdentDelivery.cpp:99-180): GSyn[b][k] += A_ext[b][kex(k)] for
 * every restricted neuron k of an IdentConn (pre and post of the same size).  Sparse form when
 * entries != NULL (halo entries skipped), dense form from aExt otherwise; gsyn is the channel's
 * [nbatch][ny][nx][nf] buffer. */
pvgpu_status pvgpu_deliver_ident(const pvgpu_loc *pre, const pvgpu_loc *post, const pvgpu_entry *entries,
                                 const int64_t *numActive, const float *aExt, float *gsyn, void *stream);
/* ErrScaleInternalStateBuffer::updateBufferCPU (components/ErrScaleInternalStateBuffer.cpp:41-53):
 * V[k] *= errScale for the n neurons across the batch (after V = accumulated GSyn). */
pvgpu_status pvgpu_err_scale(int64_t n, float errScale, float *v, void *stream);


/* ---- a6..a9: layer update ------------------------------------------------------------- */
/* updateGSynAccumulatorOnGPU (components/GSynAccumulator.kpp:16-44): G = sum_ch coeff[ch]*GSyn[ch].
 * coeffs is a host array of numChannels floats. */
pvgpu_status pvgpu_gsyn_accumulate(
      int64_t numNeuronsAcrossBatch,
      int numChannels,
      const float *coeffs,
      const float *gsyn,
      float *g,
      void *stream);

/* updateHyPerLCAOnGPU (components/HyPerLCAInternalStateBuffer.kpp:18-63):
 * V = e*V + (1-e)*(G + selfInteract*A_ext), e = (float)exp(-dtAdapt[b]/tau).  dtAdapt is a
 * device array of nbatch doubles.  Products and sums are rounded as the CPU path rounds them. */
pvgpu_status pvgpu_lca_update(
      const pvgpu_loc *loc,
      int selfInteract,
      const double *dtAdapt,
      float tau,
      const float *g,
      const float *aExt,
      float *v,
      void *stream);

/* MomentumLCAInternalStateBuffer::updateBufferGPU / updateMomentumLCAOnGPU
 * (components/MomentumLCAInternalStateBuffer.kpp:18-69): drive = (1 - e)(G + selfInteract A),
 * V = e V + drive + momentumRate prevDrive, prevDrive = drive; e = (float)exp(-dtAdapt[b]/tau).
 * Bit-identical to the reference CPU update. */
pvgpu_status pvgpu_momentum_lca_update(const pvgpu_loc *loc, int selfInteract, float momentumRate,
                                       const double *dtAdapt, float tau, const float *g, const float *aExt,
                                       float *prevDrive, float *v, void *stream);
/* ISTAInternalStateBuffer::updateBufferGPU / updateISTAInternalStateBufferOnGPU
 * (components/ISTAInternalStateBuffer.kpp:16-63): V += ((float)dtAdapt[b] / tau)(G - VThresh sign(A)).
 * Bit-identical to the reference CPU update. */
pvgpu_status pvgpu_ista_update(const pvgpu_loc *loc, float VThresh, const double *dtAdapt, float tau, const float *g,
                               const float *aExt, float *v, void *stream);


/* ANNActivityBuffer threshold, CPU form (components/ANNActivityBuffer.cpp:432-558; the
 * reference GPU runs the vertex form of ANNActivityBuffer.kpp:16-77 instead): A_ext = T(V) on
 * the restricted region; the halo is left untouched. */
pvgpu_status pvgpu_ann_activity(
      const pvgpu_loc *loc,
      const float *v,
      float VThresh,
      float AMin,
      float AMax,
      float AShift,
      float VWidth,
      float *aExt,
      void *stream);

/* applyVerticesANNActivityBufferOnGPU (components/ANNActivityBuffer.kpp:16-77), the form the
 * reference's GPU path uses for every ANN layer and the only one for a vertex list given in
 * params (verticesV / verticesA / slopeNegInf / slopePosInf): numVertices vertices and
 * numVertices + 1 slopes (slopes[0] below the first vertex, slopes[numVertices] from the last
 * on), all device arrays.  V restricted -> A extended (halo untouched).  Products and sums
 * rounded separately, as the CPU form of the same function. */
pvgpu_status pvgpu_ann_vertices(
      const pvgpu_loc *loc,
      int numVertices,
      const float *verticesV,
      const float *verticesA,
      const float *slopes,
      const float *v,
      float *aExt,
      void *stream);

/* The three update kernels fused (HyPerActivityComponent::updateActivity,
 * components/HyPerActivityComponent.tpp:81-90, running GSynAccumulator -> HyPerLCAInternalStateBuffer
 * -> ANNActivityBuffer): one pass over the layer.  gsyn holds numChannels channels. */
typedef struct {
   pvgpu_loc loc;
   int numChannels;
   float coeffs[4];
   int selfInteract;
   float tau;
   float VThresh, AMin, AMax, AShift, VWidth;
} pvgpu_lca_layer_desc;

pvgpu_status pvgpu_lca_layer_update(
      const pvgpu_lca_layer_desc *desc,
      const float *gsyn,
      const double *dtAdapt,
      float *v,
      float *aExt,
      void *stream);

/* ---- a11: energy probes, FP64 on the device ------------------------------------------------
 * CostFunctionSum<C>::calculateSumNoMask (probes/CostFunctionSum.hpp:86-108) per batch element:
 * kind 0 = L2 (x^2), 1 = L1 (|x|), 2 = firm threshold (p0 = VThresh, p1 = VWidth,
 * probes/CostFunctions.hpp:32-49).  out: device array of nbatch doubles (overwritten).
 * Deterministic fixed-order reduction. */
pvgpu_status pvgpu_cost_sum(
      const pvgpu_loc *loc,
      const float *bufExt,
      int kind,
      double p0,
      double p1,
      double *out,
      void *stream);

/* ---- config 4: the gradient of unrolled LCA (differentiable dictionary learning) ----------
 * No single reference counterpart: the reference learns dictionaries with the Hebbian rule
 * (weightupdaters/HebbianUpdater.cpp:476-629), which is minus the gradient below for a fixed
 * activity.  L(W) = 0.5 ||x - W^T a_T||^2 + lambda ||a_T||_1 summed over the batch, a_T after
 * `steps` LCA timesteps from V = 0 (soft threshold a = max(V - VThresh, 0); V' = e V + (1 - e)
 * (W (x - W^T a) + a), e = exp(-dt / tau), the update of HyPerLCAInternalStateBuffer.kpp:18-63),
 * and dL/dW through the unrolled solve, checkpointed every `checkpointEvery` timesteps.  The V1
 * layer tiles the input with one stride S = inNx / v1Nx; patches nxp x nxp x inNf with
 * (nxp - S) even (the LCA one-to-many geometry).  W: device FP32 [v1Nf][nxp][nxp][inNf] (the
 * V1 -> error weights), x: device FP32 [nbatch][inNy][inNx][inNf]; dW (same layout as W) and
 * *loss (device double) are overwritten.  The deliveries and their adjoints are GEMMs over
 * im2col'd operands (FP32, emulated on the BF16 tensor cores where the cuBLAS in the process
 * offers it; pvgpu_lca_grad_info tells), the rest the library's own kernels; a run is one CUDA
 * graph, captured at the first run with a given set of pointers (make that run outside any
 * stream capture) and replayed on `stream`.  create returns PVGPU_ERR_UNSUPPORTED_SHAPE when
 * cuBLAS cannot be loaded. */
typedef struct {
   int nbatch, inNx, inNy, inNf;
   int v1Nx, v1Ny, v1Nf;
   int nxp;
   float VThresh, lambda1, tau, dt; /* lambda1: the L1 coefficient of the loss */
   int steps, checkpointEvery;
} pvgpu_lca_grad_desc;
typedef struct pvgpu_lca_grad pvgpu_lca_grad;
pvgpu_status pvgpu_lca_grad_create(const pvgpu_lca_grad_desc *desc, pvgpu_lca_grad **out);
pvgpu_status pvgpu_lca_grad_destroy(pvgpu_lca_grad *g);
pvgpu_status pvgpu_lca_grad_run(pvgpu_lca_grad *g, const float *w, const float *x, float *dW, double *loss,
                                void *stream);
/* *emulatedFp32 = 1 when the GEMMs run as FP32 emulated on the BF16 tensor cores, 0 for plain FP32. */
pvgpu_status pvgpu_lca_grad_info(const pvgpu_lca_grad *g, int *emulatedFp32);

/* ---- a12: Hebbian weight update and the adjoint of delivery ------------------------------
 * HebbianUpdater::update_dW / updateInd_dW (weightupdaters/HebbianUpdater.cpp:476-629), shared
 * weights, summed over the batch, normalize_dW off: dW[kernel][item] = dWMax * sum pre*post.
 * dw ([numKernels][nyp][nxp][post.nf]) is overwritten.  Deterministic (no atomics). */
pvgpu_status pvgpu_hebbian_dw(
      const pvgpu_conn_desc *conn,
      float dWMax,
      const float *preExt,
      const float *postExt,
      float *dw,
      void *stream);

/* ---- MomentumUpdater (weightupdaters/MomentumUpdater.cpp:291-345) --------------------------
 * The momentum factors of MomentumUpdater::applyMomentum for momentumMethod 'v' (viscosity:
 * dwFactor = exp(-1/tau), 0 for tau 0), 's' (simple: tau) and 'a' (alex: tau, wFactor scaled by
 * dWMax); wFactor = momentumDecay.  Host function. */
pvgpu_status pvgpu_momentum_factors(char method, float tau, float decay, float dWMax, float *dwFactor, float *wFactor);
/* One MomentumUpdater::updateWeights on the device, weight by weight: dW = dW*(1 - dwFactor)
 * + dwFactor*prev_dW - wFactor*W, then prev_dW = dW and W += dW (HebbianUpdater::updateWeights).
 * dw holds the Hebbian dW of this update (pvgpu_hebbian_dw) on entry. */
pvgpu_status pvgpu_momentum_update_weights(int64_t n, float dwFactor, float wFactor, float *dw, float *prevDw,
                                           float *w, void *stream);

/* ---- the batched LCA module ------------------------------------------------------------------
 * The per-timestep layer sequence of an LCA module (input -> error <-> V1; the LCA-CIFAR
 * topology of tutorials/LCA-CIFAR and tests/GPULCATest), replacing, per step, the reference's
 *   error layer:  IdentDelivery (ch0) + PresynapticPerspectiveConvolveDelivery of V1 (ch1),
 *                 GSynAccumulator, ErrScaleInternalStateBuffer, ANNActivityBuffer (identity);
 *   V1:           PostsynapticPerspectiveConvolveDelivery of the error (TransposeConn),
 *                 GSynAccumulator, HyPerLCAInternalStateBuffer, ANNActivityBuffer
 * driven by HyPerCol::advanceTime (columns/HyPerCol.cpp:659-790), with the host round trips of
 * the reference GPU path (datastore H->D, SparseList on the host, V/A/GSyn D->H) removed.
 * Each timestep is two fused kernels: (1) reconstruction W^T a as a GEMM + deterministic fold,
 * (2) residual + post-perspective delivery GEMM + LCA update + threshold in the epilogue.
 * Supported geometry: V1 stride S = inNx / v1Nx in {2, 4}, square patch nxp, with
 * (S, nxp, inNf) in {(2, 8, 1), (2, 8, 3), (4, 16, 1)}, v1Nx * v1Ny a multiple of 128, 128 a
 * multiple of v1Nx, v1Nf a multiple of 64. */
typedef struct {
   int nbatch;
   int inNx, inNy, inNf;   /* input / error layer, restricted */
   int v1Nx, v1Ny, v1Nf;   /* V1, restricted */
   int nxp;                /* V1 -> error patch (square), nfp = inNf */
   float VThresh, AMin, AMax, AShift, VWidth;  /* ANNActivityBuffer parameters of V1 */
   float tau;              /* timeConstantTau / dt (HyPerLCAInternalStateBuffer.cpp:104-112) */
   float dt;               /* the time step handed to the update (dtAdapt without an adaptive probe) */
   int selfInteract;
} pvgpu_lca_solver_desc;

typedef struct pvgpu_lca_solver pvgpu_lca_solver;

enum {
   PVGPU_LCA_FP32 = 0, /* FP32 SIMT GEMMs, FP32 activity: the plain form */
   PVGPU_LCA_BF16 = 1  /* tcgen05 BF16 GEMMs with FP32 accumulation, FP32 residual and V */
};

/* Allocates the solver's device state (V, activity, reconstruction partials, weight copies). */
pvgpu_status pvgpu_lca_solver_create(const pvgpu_lca_solver_desc *desc, pvgpu_lca_solver **out);
pvgpu_status pvgpu_lca_solver_destroy(pvgpu_lca_solver *s);
/* w: device FP32 [v1Nf][nxp][nxp][inNf], the V1 -> error weights (already normalised). */
pvgpu_status pvgpu_lca_solver_set_weights(pvgpu_lca_solver *s, const float *w, void *stream);
/* V = v0 (device FP32 [nbatch][v1Ny][v1Nx][v1Nf]) or zeros when v0 is NULL; A = T(V). */
pvgpu_status pvgpu_lca_solver_reset(pvgpu_lca_solver *s, const float *v0, void *stream);
/* numSteps timesteps on input x (device FP32 [nbatch][inNy][inNx][inNf]); in BF16 precision the
 * last numX3Steps run with BF16x3 split products (hi*hi + hi*lo + lo*hi). */
pvgpu_status pvgpu_lca_solver_run(pvgpu_lca_solver *s, const float *x, int numSteps, int numX3Steps, int precision,
                                  void *stream);
/* Energy of the last step as the reference's ColumnEnergyProbe computes it
 * (probes/ColumnEnergyProbe.cpp:60-70): l2Coeff * sum(err^2) (L2NormProbe) + costCoeff *
 * sum(cost(A_V1)), cost = |a| (costKind 1, L1NormLCAProbe) or the firm-threshold cost
 * (costKind 2, FirmThresholdCostFnLCAProbe); FP64, energy = device array of nbatch doubles. */
pvgpu_status pvgpu_lca_solver_energy(pvgpu_lca_solver *s, const float *x, double l2Coeff, int costKind,
                                     double costThresh, double costWidth, double costCoeff, double *energy,
                                     void *stream);
/* Copies V and/or A = T(V) (device FP32, restricted layout) out of the solver; either may be NULL. */
pvgpu_status pvgpu_lca_solver_state(pvgpu_lca_solver *s, float *v, float *a, void *stream);
/* Reads (synchronously) the solver's device error flag: nonzero if a bounded device wait gave up. */
pvgpu_status pvgpu_lca_solver_error_flag(pvgpu_lca_solver *s, int *hostFlag);
/* Per-kernel timing of the next maxSteps timesteps with CUDA events on the run's stream (the
 * counterpart of the reference's CudaTimer around recvsyn / update, arch/cuda/CudaTimer.hpp:23-63).
 * profile_end synchronises on the last event and returns the summed milliseconds of the
 * reconstruction kernel and of the post-delivery/update kernel over the recorded steps. */
pvgpu_status pvgpu_lca_solver_profile_begin(pvgpu_lca_solver *s, int maxSteps);
pvgpu_status pvgpu_lca_solver_profile_end(pvgpu_lca_solver *s, double *reconMs, double *postMs, int *steps);
/* The same split three ways: kernel R, kernel P, and the fused single-launch timesteps (kernel
 * F, see pvgpu_lca_schedule.fused), with the number of timesteps that ran kernel F. */
pvgpu_status pvgpu_lca_solver_profile_end_fused(pvgpu_lca_solver *s, double *reconMs, double *postMs,
                                                double *fusedMs, int *steps, int *fusedSteps);
/* No counterpart in the reference (its CUDA kernels have fixed launch shapes).  Times every
 * shape of the two BF16 kernels that fits in shared memory -- the post-delivery kernel's feature
 * tile (64/128/256/512) and its V / weight ring depths and A staging, the reconstruction
 * kernel's ring depth -- on trialSteps timesteps of x (BF16 and BF16x3 forms), keeps the fastest
 * of each, then replays graphs of max(trialSteps, 16) steps under each schedule (one chain or two
 * half-batch chains, with and without programmatic edges, two chains with capped grids for
 * kernels P and F: pvgpu_lca_solver_set_schedule) and keeps the fastest; remembers shapes and schedule for every solver of the same geometry created later
 * in the process.  Leaves V and A undefined: call pvgpu_lca_solver_reset before the next run. */
pvgpu_status pvgpu_lca_solver_autotune(pvgpu_lca_solver *s, const float *x, int trialSteps, void *stream);
/* The shapes in use: out[0..4] = {feature tile, V ring slots, weight ring slots, A staged (0/1),
 * reconstruction ring stages} of the BF16 form, out[5..9] the same for BF16x3 steps. */
pvgpu_status pvgpu_lca_solver_plan_info(const pvgpu_lca_solver *s, int *out);
/* The fused kernel's shape: out[0..2] = {feature tile, V ring slots, weight ring slots}, zeros
 * when the geometry has no fused form. */
pvgpu_status pvgpu_lca_solver_fused_plan_info(const pvgpu_lca_solver *s, int *out);
/* Sets the fused kernel's shape (what the autotuner otherwise picks): feature tile (a multiple
 * of 64 dividing v1Nf), V ring slots (2 or 4), weight ring slots (2..4); PVGPU_ERR_UNSUPPORTED_SHAPE
 * when it does not fit shared memory.  The ring depths do not change results; the feature tile
 * sets how the reconstruction is split into bands (FP32 summation order of the residual). */
pvgpu_status pvgpu_lca_solver_set_fused_plan(pvgpu_lca_solver *s, int featureTile, int vSlots, int wSlots);

/* No counterpart in the reference.  How a BF16 run is laid out: fused = 1 runs the BF16
 * timesteps as one launch each (kernel F: post delivery, update and the reconstruction of the
 * new activity, which stays on chip; each block's reconstruction leaves as a band of padded rows
 * that the next step's windows sum) except the run's first (kernel R then F) and its final BF16
 * step and BF16x3 steps (kernels R and P); fused = 0 runs kernels R and P on every step.  The
 * two forms differ only in FP32 summation order of the residual.  chains = 1 runs the whole
 * batch as one chain of kernels; chains = 2 runs the two halves of the batch (images [0, n0)
 * and [n0, nbatch), n0 = nbatch / 2 rounded up to even when that leaves images for the second
 * half) as two independent chains on parallel graph branches, so that the kernels of one half
 * run in the ramp and tail of the other's.  reconCtas / postCtas cap the persistent grids of
 * kernel R (rounded down to clusters of two) and of kernels P and F (0 = as many as fit).
 * programmatic = 1 launches each kernel of a chain early (programmatic stream serialisation) so
 * that its set-up overlaps the kernel before it.  chains, the caps and programmatic do not
 * change the results.  Default {1, 0, 0, 1, 1}; per-kernel profiling runs use one chain. */
typedef struct {
   int chains;
   int reconCtas;
   int postCtas;
   int programmatic;
   int fused;
} pvgpu_lca_schedule;
pvgpu_status pvgpu_lca_solver_set_schedule(pvgpu_lca_solver *s, const pvgpu_lca_schedule *sc);
pvgpu_status pvgpu_lca_solver_get_schedule(const pvgpu_lca_solver *s, pvgpu_lca_schedule *sc);

/* ---- diagnostics ----------------------------------------------------------------------------
 * No counterpart in the reference.  C[M][N] (FP32) = A[M][K] * B[N][K]^T with BF16 row-major
 * operands on the tcgen05 tensor cores through TMA and TMEM: the building block of the BF16
 * LCA kernels, exposed so a test can check it against a host GEMM.  M % 128 == 0,
 * 16 <= N <= 256 with N % 16 == 0, K % 64 == 0; A, B 16-byte aligned.  *errFlag (device int)
 * is set to 1 if a bounded device wait gave up. */
pvgpu_status pvgpu_tc_gemm_bf16(const void *A, const void *B, float *C, int M, int N, int K, int *errFlag, void *stream);
/* The same with B given as [K][N] (N contiguous, N % 64 == 0), read by the MMA as an MN-major
 * operand: C = A * B. */
pvgpu_status pvgpu_tc_gemm_bf16_kn(const void *A, const void *B, float *C, int M, int N, int K, int *errFlag,
                                   void *stream);
/* The same as pvgpu_tc_gemm_bf16 with A read by the MMA from tensor memory (each row stored into
 * its TMEM lane, two K elements per column); 64 <= K <= 256. */
pvgpu_status pvgpu_tc_gemm_bf16_atmem(const void *A, const void *B, float *C, int M, int N, int K, int *errFlag,
                                      void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PVGPU_H_ */
