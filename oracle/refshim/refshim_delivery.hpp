// refshim_delivery.hpp -- minimal stand-ins for the OpenPV framework classes that the
// reference's delivery translation units (delivery/PresynapticPerspectiveConvolveDelivery.cpp,
// delivery/PostsynapticPerspectiveConvolveDelivery.cpp) refer to, so that those files compile
// unmodified, where they lie, into oracle/_ref.  TEST INFRASTRUCTURE ONLY.
//
// Only the members the two deliver() loops use exist here: layer locations, the presynaptic
// activity cube (dense data + SparseList), one arbor with delay 0, and shared weights whose
// patch tables come from the reference's own PatchGeometry (compiled from its source).
#pragma once

#include "components/PatchGeometry.hpp"
#include "include/PVLayerLoc.h"
#include "include/pv_types.h"
#include "structures/Patch.hpp"
#include "structures/SparseList.hpp"
#include "utils/PVAssert.hpp"
#include "utils/conversions.hpp"

#include <memory>
#include <string>
#include <vector>

namespace PV {

class PVParams;
class Communicator;
struct CommunicateInitInfoMessage {};

namespace Response {
enum Status { SUCCESS, NO_ACTION, PARTIAL, POSTPONE };
inline bool completed(Status s) { return s == SUCCESS || s == NO_ACTION; }
}  // namespace Response

class BaseObject {
  public:
   virtual ~BaseObject() {}
   void initialize(char const *, PVParams *, Communicator const *) { setObjectType(); }
   virtual void setObjectType() {}

  protected:
   std::string mObjectType;
};

// Shared weights over a PatchGeometry: data [kernel][nyp][nxp][nfp].
class Weights {
  public:
   Weights(PVLayerLoc const &pre, PVLayerLoc const &post, int nxp, int nyp, float const *data)
         : mPre(pre), mPost(post) {
      mGeometry = std::make_shared<PatchGeometry>("refshim", nxp, nyp, post.nf, &pre, &post);
      mGeometry->allocateDataStructures();
      mNkx = pre.nx > post.nx ? pre.nx / post.nx : 1;
      mNky = pre.ny > post.ny ? pre.ny / post.ny : 1;
      mNkf = pre.nf;
      mData.assign(data, data + (size_t)mNkx * mNky * mNkf * nxp * nyp * post.nf);
   }
   std::shared_ptr<PatchGeometry> getGeometry() const { return mGeometry; }
   Patch const &getPatch(int k) const { return mGeometry->getPatch(k); }
   int getPatchSizeX() const { return mGeometry->getPatchSizeX(); }
   int getPatchSizeY() const { return mGeometry->getPatchSizeY(); }
   int getPatchSizeF() const { return mGeometry->getPatchSizeF(); }
   int getPatchStrideY() const { return mGeometry->getPatchStrideY(); }
   // the kernel of an extended presynaptic index (shared weights)
   float *getDataFromPatchIndex(int arbor, int patchIndex) {
      (void)arbor;
      int npx = mPre.nx + mPre.halo.lt + mPre.halo.rt, npy = mPre.ny + mPre.halo.dn + mPre.halo.up;
      int x = (kxPos(patchIndex, npx, npy, mPre.nf) - mPre.halo.lt) % mNkx;
      if (x < 0) x += mNkx;
      int y = (kyPos(patchIndex, npx, npy, mPre.nf) - mPre.halo.up) % mNky;
      if (y < 0) y += mNky;
      int kernel = kIndex(x, y, featureIndex(patchIndex, npx, npy, mPre.nf), mNkx, mNky, mNkf);
      return mData.data() + (size_t)kernel * mGeometry->getPatchSizeOverall();
   }

  private:
   PVLayerLoc mPre, mPost;
   std::shared_ptr<PatchGeometry> mGeometry;
   int mNkx, mNky, mNkf;
   std::vector<float> mData;
};

class WeightsPair {
  public:
   Weights *pre = nullptr, *post = nullptr;
   bool getInitInfoCommunicatedFlag() const { return true; }
   void needPre() {}
   void needPost() {}
   Weights *getPreWeights() { return pre; }
   Weights *getPostWeights() { return post; }
};

class ArborList {
  public:
   int getNumAxonalArbors() const { return 1; }
   int getDelay(int) const { return 0; }
};

class Publisher {
  public:
   PVLayerCube cube;
   PVLayerCube createCube(int) const { return cube; }
};

class PreData {
  public:
   PVLayerLoc loc;
   bool sparse = false;
   Publisher publisher;
   PVLayerLoc const *getLayerLoc() const { return &loc; }
   bool getSparseLayer() const { return sparse; }
   Publisher *getPublisher() { return &publisher; }
};

class PostGSyn {
  public:
   PVLayerLoc loc;
   PVLayerLoc const *getLayerLoc() const { return &loc; }
   int getBufferSize() const { return loc.nx * loc.ny * loc.nf; }
};

class HyPerDelivery : public BaseObject {
  public:
   virtual void deliver(float *destBuffer)      = 0;
   virtual void deliverUnitInput(float *buffer) = 0;
   int getChannelCode() const { return mChannelCode; }
   void wire(PreData *pre, PostGSyn *post, WeightsPair *wp, ArborList *arbors) {
      mPreData     = pre;
      mPostGSyn    = post;
      mWeightsPair = wp;
      mArborList   = arbors;
   }

  protected:
   virtual Response::Status communicateInitInfo(std::shared_ptr<CommunicateInitInfoMessage const>) {
      return Response::SUCCESS;
   }
   virtual Response::Status allocateDataStructures() { return Response::SUCCESS; }
   float *setWorkingGSynBuffer(float *b) { return b; }
   void accumulateThreadGSyn(float *) {}

   bool mReceiveGpu        = false;
   float mDeltaTimeFactor  = 1.0f;
   int mChannelCode        = CHANNEL_EXC;
   PreData *mPreData       = nullptr;
   PostGSyn *mPostGSyn     = nullptr;
   WeightsPair *mWeightsPair = nullptr;
   ArborList *mArborList   = nullptr;
};

}  // namespace PV
