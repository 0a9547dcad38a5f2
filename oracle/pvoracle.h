/*
 * pvoracle.h -- CPU restatement of OpenPV's synaptic-delivery + LCA-update path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the GPU path in
 * openpv_gb300 is compared against.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py may load it.  The product path never
 * links, loads or calls it.
 *
 * Every function restates one loop of the reference and cites the reference file
 * and line it follows (paths are relative to the OpenPV source tree).  Summation
 * order follows the reference's single-thread (-t 1) order so that the float
 * variants agree bit for bit with the reference CPU path; the *_f64 variants keep
 * the same algorithm in double precision and serve as the FP64 oracle.
 *
 * Parity of this restatement is pinned by:
 *   - oracle/_ref: the reference's own PatchGeometry.cpp and its .kpp update
 *     kernels (HyPerLCAInternalStateBuffer.kpp, GSynAccumulator.kpp,
 *     ANNActivityBuffer.kpp) compiled from the reference tree and compared
 *     bit-exactly (tests/test_oracle_vs_ref.py);
 *   - the reference's golden LCA reconstruction (tests/GPULCATest/input/correct.pvp,
 *     with weights.pvp, initialV1.pvp and inputImages.pvp) reproduced by
 *     pvo_lca_run() (tests/test_oracle_golden.py).
 */
#ifndef PVORACLE_H_
#define PVORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors PVHalo / PVLayerLoc (include/PVLayerLoc.h:14-26), batch-local fields only. */
typedef struct {
   int lt, rt, dn, up;
} pvo_halo;

typedef struct {
   int nbatch, nx, ny, nf;
   pvo_halo halo;
} pvo_loc;

/* Mirrors Patch (structures/Patch.hpp:15-18). */
typedef struct {
   uint16_t nx, ny;
   uint32_t offset;
} pvo_patch;

/* Mirrors SparseList<float>::Entry (structures/SparseList.hpp:19-22). */
typedef struct {
   uint32_t index;
   float value;
} pvo_entry;

/* ---- geometry ---------------------------------------------------------- */

/* utils/requiredConvolveMargin.hpp; returns -1 on an illegal geometry. */
int pvo_required_margin(int nPre, int nPost, int patchSize);
/* PatchSize::calcPostPatchSize (components/PatchSize.cpp:98-130); -1 if illegal. */
int pvo_post_patch_size(int prePatchSize, int nPre, int nPost);

/* PatchGeometry::setPatchGeometry (components/PatchGeometry.cpp:179-262).
 * Arrays have numPatches = nxExt(pre) * nyExt(pre) * nf(pre) entries.  Any output
 * pointer may be NULL.  Returns 0, or -1 on an illegal geometry. */
int pvo_patch_geometry(
      const pvo_loc *pre,
      const pvo_loc *post,
      int nxp,
      int nyp,
      pvo_patch *patches,
      int64_t *gSynPatchStart,
      int64_t *aPostOffset,
      int64_t *unshrunkenStart);

/* Weights::calcDataIndexFromPatchIndex for shared weights (components/Weights.cpp:208-232):
 * table[kPreExt] = kernel index.  Returns the number of kernels. */
int pvo_kernel_index_table(const pvo_loc *pre, const pvo_loc *post, int32_t *table);

/* PatchGeometry::setTransposeItemIndices (components/PatchGeometry.cpp:264-332) followed by
 * TransposeWeights::transposeShared (utils/TransposeWeights.cpp:56-115): fills the post
 * weights (kernels of the post->pre geometry, patch nxpPost x nypPost x pre.nf).
 * Returns 0 or -1. */
int pvo_transpose_shared(
      const pvo_loc *pre,
      const pvo_loc *post,
      int nxp,
      int nyp,
      const float *wPre,
      float *wPost);

/* ---- a1: active-index compaction ----------------------------------------- */
/* DataStore::updateActiveIndices (columns/DataStore.cpp:46-66), per batch element.
 * entries: [nbatch][numExt] capacity; numActive: [nbatch] (long in the reference). */
void pvo_compact(const float *aExt, int nbatch, int numExt, pvo_entry *entries, int64_t *numActive);

/* ---- a4: presynaptic-perspective convolve delivery ----------------------- */
/* PresynapticPerspectiveConvolveDelivery::deliver (delivery/PresynapticPerspectiveConvolveDelivery.cpp:61-192),
 * single arbor, shared weights.  If entries != NULL the sparse branch runs (entries/numActive per batch,
 * stride numPreExt); otherwise the dense branch reads aExt.  gsyn ([nbatch][post restricted]) is
 * accumulated into, not cleared. */
int pvo_deliver_pre(
      const pvo_loc *pre,
      const pvo_loc *post,
      int nxp,
      int nyp,
      const float *w,
      const pvo_entry *entries,
      const int64_t *numActive,
      const float *aExt,
      float dtFactor,
      float *gsyn);
int pvo_deliver_pre_f64(
      const pvo_loc *pre,
      const pvo_loc *post,
      int nxp,
      int nyp,
      const double *w,
      const double *aExt,
      double dtFactor,
      double *gsyn);

/* ---- a5: postsynaptic-perspective convolve delivery ---------------------- */
/* PostsynapticPerspectiveConvolveDelivery::deliver (delivery/PostsynapticPerspectiveConvolveDelivery.cpp:56-151).
 * src = presynaptic layer (activity aExt, extended), tgt = layer receiving GSyn.  wPost holds the
 * post-perspective weights: kernels of the tgt->src geometry with patch nxpPost x nypPost x src.nf. */
int pvo_deliver_post(
      const pvo_loc *src,
      const pvo_loc *tgt,
      int nxpPost,
      int nypPost,
      const float *wPost,
      const float *aExt,
      float dtFactor,
      float *gsyn);
int pvo_deliver_post_f64(
      const pvo_loc *src,
      const pvo_loc *tgt,
      int nxpPost,
      int nypPost,
      const double *wPost,
      const double *aExt,
      double dtFactor,
      double *gsyn);

/* ---- a6..a9: layer update ------------------------------------------------ */
/* GSynAccumulator.kpp:16-44 */
void pvo_gsyn_accumulate(int numNeuronsAcrossBatch, int numChannels, const float *coeffs, const float *gsyn, float *g);
/* MomentumLCAInternalStateBuffer.kpp:18-69 */
void pvo_momentum_lca_update(const pvo_loc *loc, int selfInteract, float momentumRate, const double *dtAdapt, float tau,
                             const float *g, const float *aExt, float *prevDrive, float *v);
void pvo_momentum_lca_update_f64(const pvo_loc *loc, int selfInteract, double momentumRate, const double *dtAdapt,
                                 double tau, const double *g, const double *aExt, double *prevDrive, double *v);
/* ISTAInternalStateBuffer.kpp:16-63 */
void pvo_ista_update(const pvo_loc *loc, float VThresh, const double *dtAdapt, float tau, const float *g,
                     const float *aExt, float *v);
void pvo_ista_update_f64(const pvo_loc *loc, double VThresh, const double *dtAdapt, double tau, const double *g,
                         const double *aExt, double *v);
/* HyPerLCAInternalStateBuffer.kpp:18-63 */
void pvo_lca_update(
      const pvo_loc *loc,
      int selfInteract,
      const double *dtAdapt,
      float tau,
      const float *g,
      const float *aExt,
      float *v);
void pvo_lca_update_f64(
      const pvo_loc *loc,
      int selfInteract,
      const double *dtAdapt,
      double tau,
      const double *g,
      const double *aExt,
      double *v);
/* HyPerActivityBuffer::updateBufferCPU (components/HyPerActivityBuffer.cpp:36-54) then
 * ANNActivityBuffer::applyVThresh / applyAMax (components/ANNActivityBuffer.cpp:490-558). */
void pvo_ann_activity(
      const pvo_loc *loc,
      const float *v,
      float VThresh,
      float AMin,
      float AMax,
      float AShift,
      float VWidth,
      float *aExt);
void pvo_ann_activity_f64(
      const pvo_loc *loc,
      const double *v,
      double VThresh,
      double AMin,
      double AMax,
      double AShift,
      double VWidth,
      double *aExt);
/* ANNActivityBuffer::setVertices / setSlopes (components/ANNActivityBuffer.cpp:227-400) followed by the
 * vertex transfer function of ANNActivityBuffer.kpp:16-77 (the reference's GPU form).  Returns the
 * number of vertices (<= 4) written to vV/vA and slopes (numVertices + 1). */
int pvo_ann_vertices(
      float VThresh,
      float AMin,
      float AMax,
      float AShift,
      float VWidth,
      float *vV,
      float *vA,
      float *slopes);

/* ---- a11: energy terms ---------------------------------------------------- */
/* CostFunctionSum<C>::calculateSumNoMask (probes/CostFunctionSum.hpp:86-108) per batch element, double
 * accumulation in neuron order.  kind: 0 = L2 (x*x), 1 = L1 (|x|), 2 = firm threshold (CostFunctions.hpp:32-49). */
void pvo_cost_sum(const pvo_loc *loc, const float *bufExt, int kind, double p0, double p1, double *out);
void pvo_cost_sum_f64(const pvo_loc *loc, const double *bufExt, int kind, double p0, double p1, double *out);

/* AdaptiveTimeScaleController::calcTimesteps (components/AdaptiveTimeScaleController.cpp:57-86).
 * state: [nbatch][3] = {timeScale, timeScaleMax, timeScaleTrue}. */
void pvo_adaptive_timescale(
      int nbatch,
      double baseMax,
      double baseMin,
      double tauFactor,
      double growthFactor,
      const double *energies,
      double *state);

/* ---- a12: Hebbian weight update ------------------------------------------ */
/* HebbianUpdater::update_dW / updateInd_dW (weightupdaters/HebbianUpdater.cpp:476-629) for shared
 * weights, one arbor, convolve accumulation, summed over the batch; normalize_dW off.
 * dw ([numKernels][nyp][nxp][post.nf]) is overwritten. */
int pvo_hebbian_dw(
      const pvo_loc *pre,
      const pvo_loc *post,
      int nxp,
      int nyp,
      float dWMax,
      const float *preExt,
      const float *postExt,
      float *dw);
int pvo_hebbian_dw_f64(
      const pvo_loc *pre,
      const pvo_loc *post,
      int nxp,
      int nyp,
      double dWMax,
      const double *preExt,
      const double *postExt,
      double *dw);
/* The same loop with the update rule chosen (0: dWMax * pre * post; 1: pre - post, the rule of
 * the reference's PlasticConnTest updater) and, when counts is not NULL, the number of
 * contributions per kernel item (the divisor of HebbianUpdater::normalize_dW). */
int pvo_hebbian_dw_rule(
      const pvo_loc *pre,
      const pvo_loc *post,
      int nxp,
      int nyp,
      int rule,
      float dWMax,
      const float *preExt,
      const float *postExt,
      float *dw,
      int64_t *counts);
int pvo_hebbian_dw_rule_f64(
      const pvo_loc *pre,
      const pvo_loc *post,
      int nxp,
      int nyp,
      int rule,
      double dWMax,
      const double *preExt,
      const double *postExt,
      double *dw,
      int64_t *counts);

/* ---- the canonical LCA module -------------------------------------------- */
/* Input -> Error (IdentConn ch0), V1 -> Error (pre perspective, sparse, ch1),
 * Error -> V1 (TransposeConn, post perspective, ch0), with the phase order of
 * HyPerCol::advanceTime (columns/HyPerCol.cpp:659-790): the error layer sees the
 * input of this step and the reconstruction of the previous step; V1 sees this
 * step's error.  Matches tests/GPULCATest/input/GPULCATest.params and the
 * LCA-CIFAR topology. */
typedef struct {
   int nbatch;
   int inNx, inNy, inNf;      /* input / error layer, restricted */
   int v1Nx, v1Ny, v1Nf;      /* V1 layer, restricted */
   int nxp, nyp;              /* V1 -> Error patch (nfp = inNf) */
   float VThresh, AMin, AMax, AShift, VWidth;
   float tau;                 /* timeConstantTau / dt */
   int selfInteract;
   float errScale;
   /* adaptive time scale (AdaptiveTimeScaleProbe); adaptive = 0 uses dtFixed */
   int adaptive;
   double baseMax, baseMin, tauFactor, growthFactor;
   double dtFixed;
   int displayPeriod;         /* input frame period; the time-scale trigger fires on input updates */
   /* energy = l2Coeff * sum(err^2) + costCoeff * sum(cost(A_V1)), ColumnEnergyProbe.cpp:60-70 */
   double l2Coeff;            /* L2NormProbe coefficient (0.5 in the LCA tutorials) */
   int costKind;              /* 1 = L1 (L1NormLCAProbe), 2 = firm threshold (FirmThresholdCostFnLCAProbe) */
   double costThresh, costWidth; /* firm-threshold cost parameters (the probe's own VThresh/VWidth, double) */
   double costCoeff;          /* the LCA probes' coefficient: the layer's float VThresh widened to double */
} pvo_lca_params;

/* Runs numSteps timesteps starting at t = 1.
 *   w:        V1->Error kernels [v1Nf][nyp][nxp][inNf] (already normalised)
 *   frames:   [numFrames][nbatch][inNy][inNx][inNf]; frame k is shown for steps
 *             k*displayPeriod+1 .. (k+1)*displayPeriod (cyclic); displayPeriod <= 0 shows frame 0
 *   v1:       in/out V of V1, restricted [nbatch][v1Ny][v1Nx][v1Nf]; A is initialised from it
 *   recon:    out, [numSteps][nbatch][inNy][inNx][inNf] reconstruction after each step (may be NULL)
 *   energy:   out, [numSteps][nbatch] total energy after each step (may be NULL)
 *   aFinal:   out, final V1 activity restricted (may be NULL)
 * numThreads > 1 splits the batch across OpenMP threads (results do not depend on it).
 * Returns 0, or -1 on an illegal geometry. */
int pvo_lca_run(
      const pvo_lca_params *p,
      const float *w,
      const float *frames,
      int numFrames,
      int numSteps,
      float *v1,
      float *recon,
      double *energy,
      float *aFinal,
      int numThreads);
int pvo_lca_run_f64(
      const pvo_lca_params *p,
      const double *w,
      const double *frames,
      int numFrames,
      int numSteps,
      double *v1,
      double *recon,
      double *energy,
      double *aFinal,
      int numThreads);


/* ---- LIF (components/LIFActivityComponent.cpp:332-942) ---- */
/* taus_uint4 (include/pv_types.h:54-59): last output, then the three generator words. */
typedef struct {
   uint32_t s0, s1, s2, s3;
} pvo_taus;

/* LIFParams (components/LIFActivityComponent.hpp:22-45), same order; defaults from
 * include/default_params.h. */
typedef struct {
   float Vrest, Vexc, Vinh, VinhB;
   float VthRest, tau, tauVth, deltaVth, deltaGIB;
   float noiseAmpE, noiseAmpI, noiseAmpIB, noiseFreqE, noiseFreqI, noiseFreqIB;
   float tauE, tauI, tauIB;
} pvo_lif_params;

void pvo_taus_init(pvo_taus *state, size_t count, uint32_t seed);
void pvo_taus_next(pvo_taus *state, size_t count);
/* method 'a' (arma), 'b' (beginning: Heun), 'o' (original: Euler); returns -1 otherwise. */
int pvo_lif_update(char method, const pvo_loc *loc, const pvo_lif_params *p, float dt, pvo_taus *rnd, float *V,
                   float *Vth, float *GE, float *GI, float *GIB, const float *gsynHead, float *aExt);

/* ---- MomentumUpdater (weightupdaters/MomentumUpdater.cpp:291-345) ---- */
/* method 'v' viscosity, 's' simple, 'a' alex; -1 otherwise. */
int pvo_momentum_factors(char method, float tau, float decay, float dWMax, float *dwFactor, float *wFactor);
void pvo_momentum_update_weights(int64_t n, float dwFactor, float wFactor, float *dw, float *prevDw, float *w);

#ifdef __cplusplus
}
#endif

#endif /* PVORACLE_H_ */
