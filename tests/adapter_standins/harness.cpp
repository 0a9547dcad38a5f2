// harness.cpp -- drives the adapters of adapters/ (compiled unchanged against the stand-ins in
// this folder) through the framework's life cycle on device buffers the test owns:
// communicateInitInfo -> setCudaDevice -> allocateDataStructures -> copyInitialStateToGPU ->
// deliver, or runKernel() for the update components.  Each entry returns 0, or 1 after a
// Fatal() (the message is in standin_last_error()).  TEST INFRASTRUCTURE ONLY.
#include "components/ANNActivityBuffer.hpp"
#include "components/GSynAccumulator.hpp"
#include "components/HyPerLCAInternalStateBuffer.hpp"
#include "delivery/PostsynapticPerspectiveGPUDelivery.hpp"
#include "delivery/PresynapticPerspectiveGPUDelivery.hpp"

#include <cstring>
#include <string>

namespace PV {
struct Wiring {
   static void device(BaseObject &o, PVCuda::CudaDevice *d) {
      o.mCudaDevice   = d;
      o.mUsingGPUFlag = true;
   }
   static void delivery(HyPerDelivery &d, BasePublisherComponent *pre, LayerInputBuffer *post, WeightsPair *wp,
                        ArborList *arbors, int channel, float dtFactor) {
      d.mPreData         = pre;
      d.mPostGSyn        = post;
      d.mWeightsPair     = wp;
      d.mArborList       = arbors;
      d.mChannelCode     = (ChannelType)channel;
      d.mDeltaTimeFactor = dtFactor;
   }
};
} // namespace PV

namespace {

std::string g_error;

PVLayerLoc loc_of(const int *l8) {
   PVLayerLoc l{};
   l.nbatch = l8[0];
   l.nx     = l8[1];
   l.ny     = l8[2];
   l.nf     = l8[3];
   l.halo   = PVHalo{l8[4], l8[5], l8[6], l8[7]};
   l.nbatchGlobal = l.nbatch;
   l.nxGlobal     = l.nx;
   l.nyGlobal     = l.ny;
   return l;
}

size_t num_ext(const PVLayerLoc &l) {
   return (size_t)(l.nx + l.halo.lt + l.halo.rt) * (l.ny + l.halo.dn + l.halo.up) * l.nf;
}

template <class F>
int guarded(F &&f) {
   try {
      f();
      if (cudaDeviceSynchronize() != cudaSuccess) {
         g_error = "CUDA error after the adapter call";
         return 2;
      }
      return 0;
   } catch (PVStandin::FatalError const &e) {
      g_error = e.what();
      return 1;
   }
}

template <class D>
void life_cycle(D &d, PVCuda::CudaDevice *dev) {
   auto info = std::make_shared<PV::CommunicateInitInfoMessage const>();
   d.communicateInitInfo(info);
   auto setDev = std::make_shared<PV::SetCudaDeviceMessage const>(PV::SetCudaDeviceMessage{dev});
   d.setCudaDevice(setDev);
   d.allocateDataStructures();
   d.copyInitialStateToGPU();
}

} // namespace

extern "C" const char *standin_last_error() { return g_error.c_str(); }

// Presynaptic delivery: weights [numArbors][numKernels][nyp][nxp][post nf] on the device; GSyn
// [channels][nbatch][post restricted] on the device, channel `channel` accumulated into.  With
// hostStale, the datastore / SparseList come from the host arrays (the framework's copy path).
extern "C" int standin_pre_delivery(const int *pre8, const int *post8, int nxp, int nyp, int numKernels, int sparse,
                                    int shared, int channel, int numArbors, float dtFactor, int hostStale,
                                    float *dAext, void *dEntries, long *dNumActive, float *dW, float *dGSyn,
                                    const float *hAext, const long *hNumActive, const void *hEntries, void *stream) {
   return guarded([&] {
      PVCuda::CudaDevice dev(static_cast<cudaStream_t>(stream));
      PV::BasePublisherComponent pre;
      pre.loc     = loc_of(pre8);
      pre.sparse  = sparse != 0;
      pre.updated = hostStale != 0;
      const size_t nExt = num_ext(pre.loc);
      PVCuda::CudaBuffer ds(dAext, nExt * pre.loc.nbatch * sizeof(float));
      PVCuda::CudaBuffer ai(dEntries, nExt * pre.loc.nbatch * 8);
      PVCuda::CudaBuffer na(dNumActive, pre.loc.nbatch * sizeof(long));
      pre.datastore     = &ds;
      pre.activeIndices = sparse ? &ai : nullptr;
      pre.numActive     = sparse ? &na : nullptr;
      pre.publisher.cube.data          = hAext;
      pre.publisher.cube.loc           = pre.loc;
      pre.publisher.cube.isSparse      = sparse;
      pre.publisher.cube.numActive     = hNumActive;
      pre.publisher.cube.activeIndices = hEntries;
      PV::LayerInputBuffer post;
      post.loc = loc_of(post8);
      PVCuda::CudaBuffer gs(dGSyn, 0);
      post.cudaBuffer = &gs;
      PV::Weights w;
      w.nxp = nxp;
      w.nyp = nyp;
      w.nfp = post.loc.nf;
      w.numDataPatches = numKernels;
      w.shared         = shared != 0;
      PVCuda::CudaBuffer wd(dW, 0);
      w.deviceData = &wd;
      PV::WeightsPair wp;
      wp.pre = &w;
      PV::ArborList arbors;
      arbors.delays.assign(numArbors, 0);
      PV::PresynapticPerspectiveGPUDelivery d("standin pre delivery", nullptr, nullptr);
      PV::Wiring::delivery(d, &pre, &post, &wp, &arbors, channel, dtFactor);
      life_cycle(d, &dev);
      d.deliver(nullptr);
      if (pre.updated) throw PVStandin::FatalError("the adapter left the datastore marked stale");
   });
}

// Postsynaptic delivery: the connection pre -> post has presynaptic patch nxp x nyp; the post
// weights [numArbors][numPostKernels][nypPost][nxpPost][pre nf] are on the device.
extern "C" int standin_post_delivery(const int *pre8, const int *post8, int nxp, int nyp, int nxpPost, int nypPost,
                                     int numPostKernels, int channel, int numArbors, float dtFactor, float *dAext,
                                     float *dWpost, float *dGSyn, int *usedWorkspace, void *stream) {
   return guarded([&] {
      PVCuda::CudaDevice dev(static_cast<cudaStream_t>(stream));
      PV::BasePublisherComponent pre;
      pre.loc = loc_of(pre8);
      PVCuda::CudaBuffer ds(dAext, num_ext(pre.loc) * pre.loc.nbatch * sizeof(float));
      pre.datastore = &ds;
      PV::LayerInputBuffer post;
      post.loc = loc_of(post8);
      PVCuda::CudaBuffer gs(dGSyn, 0);
      post.cudaBuffer = &gs;
      PV::Weights wpre, wpost;
      wpre.nxp = nxp;
      wpre.nyp = nyp;
      wpre.nfp = post.loc.nf;
      wpost.nxp = nxpPost;
      wpost.nyp = nypPost;
      wpost.nfp = pre.loc.nf;
      wpost.numDataPatches = numPostKernels;
      PVCuda::CudaBuffer wd(dWpost, 0);
      wpost.deviceData = &wd;
      PV::WeightsPair wp;
      wp.pre  = &wpre;
      wp.post = &wpost;
      PV::ArborList arbors;
      arbors.delays.assign(numArbors, 0);
      PV::PostsynapticPerspectiveGPUDelivery d("standin post delivery", nullptr, nullptr);
      PV::Wiring::delivery(d, &pre, &post, &wp, &arbors, channel, dtFactor);
      life_cycle(d, &dev);
      *usedWorkspace = d.mCudnnGSyn != nullptr;
      d.deliver(nullptr);
   });
}

extern "C" int standin_lca_update(const int *loc8, int selfInteract, double scaledTau, double *dDtAdapt, float *dG,
                                  float *dAext, float *dV, void *stream) {
   return guarded([&] {
      PVCuda::CudaDevice dev(static_cast<cudaStream_t>(stream));
      PV::GSynAccumulator g;
      PV::ActivityBuffer a;
      PV::HyPerLCAInternalStateBuffer v;
      g.loc = a.loc = v.loc = loc_of(loc8);
      PVCuda::CudaBuffer gb(dG, 0), ab(dAext, 0), vb(dV, 0), dtb(dDtAdapt, 0);
      g.cudaBuffer = &gb;
      a.cudaBuffer = &ab;
      v.cudaBuffer = &vb;
      v.mCudaDtAdapt          = &dtb;
      v.mAccumulatedGSyn      = &g;
      v.mActivity             = &a;
      v.mSelfInteract         = selfInteract != 0;
      v.mScaledTimeConstantTau = scaledTau;
      PV::Wiring::device(v, &dev);
      v.runKernel();
   });
}

extern "C" int standin_ann_vertices(const int *loc8, int numVertices, float *dVerticesV, float *dVerticesA,
                                    float *dSlopes, float *dV, float *dAext, void *stream) {
   return guarded([&] {
      PVCuda::CudaDevice dev(static_cast<cudaStream_t>(stream));
      PV::InternalStateBuffer v;
      PV::ANNActivityBuffer a;
      v.loc = a.loc = loc_of(loc8);
      PVCuda::CudaBuffer vb(dV, 0), ab(dAext, 0), vv(dVerticesV, 0), va(dVerticesA, 0), sl(dSlopes, 0);
      v.cudaBuffer       = &vb;
      a.cudaBuffer       = &ab;
      a.mNumVertices     = numVertices;
      a.mCudaVerticesV   = &vv;
      a.mCudaVerticesA   = &va;
      a.mCudaSlopes      = &sl;
      a.mInternalState   = &v;
      PV::Wiring::device(a, &dev);
      a.runKernel();
   });
}

extern "C" int standin_gsyn_accumulate(const int *loc8, int numChannels, const float *coefficients, float *dGSyn,
                                       float *dG, void *stream) {
   return guarded([&] {
      PVCuda::CudaDevice dev(static_cast<cudaStream_t>(stream));
      PV::LayerInputBuffer in;
      PV::GSynAccumulator g;
      in.loc = g.loc = loc_of(loc8);
      PVCuda::CudaBuffer ib(dGSyn, 0), gb(dG, 0);
      in.cudaBuffer = &ib;
      g.cudaBuffer  = &gb;
      g.mLayerInput = &in;
      g.mNumInputChannels = numChannels;
      g.mChannelCoefficients.assign(coefficients, coefficients + numChannels);
      PV::Wiring::device(g, &dev);
      g.runKernel();
   });
}
