// standin_framework.hpp -- stand-ins for the OpenPV framework classes that the adapters in
// adapters/ touch (layer buffers, publisher, weights, arbor list, CUDA device and buffer, the
// delivery and component base classes), so that the very same adapter translation units can be
// compiled and driven on a GPU host without the reference's source tree.  Only the members the adapters
// use exist; their meaning follows the reference's (columns/BaseObject.hpp,
// components/{BasePublisherComponent,ComponentBuffer,LayerInputBuffer,Weights,WeightsPair,
// ArborList}.hpp, arch/cuda/{CudaBuffer,CudaDevice}.hpp, delivery/HyPerDelivery.hpp).  Buffers
// wrap device memory the test owns.  TEST INFRASTRUCTURE ONLY.
#pragma once

#include "include/PVLayerLoc.h"
#include "include/pv_types.h"
#include "structures/Patch.hpp"
#include "structures/SparseList.hpp"
#include "utils/PVLog.hpp"

#include <cuda_runtime_api.h>

#include <memory>
#include <string>
#include <vector>

namespace PVCuda {

class CudaBuffer {
  public:
   CudaBuffer(void *p, size_t bytes, bool owned = false) : d_ptr(p), mSize(bytes), mOwned(owned) {}
   ~CudaBuffer() {
      if (mOwned) cudaFree(d_ptr);
   }
   int copyToDevice(const void *h_ptr) {
      return cudaMemcpy(d_ptr, h_ptr, mSize, cudaMemcpyHostToDevice) == cudaSuccess ? 0 : 1;
   }
   void *getPointer() { return d_ptr; }
   size_t getSize() { return mSize; }

  private:
   void *d_ptr;
   size_t mSize;
   bool mOwned;
};

class CudaDevice {
  public:
   explicit CudaDevice(cudaStream_t s) : stream(s) {}
   cudaStream_t getStream() { return stream; }
   CudaBuffer *createBuffer(size_t bytes, std::string const *) {
      void *p = nullptr;
      if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
      return new CudaBuffer(p, bytes, true);
   }
   int get_max_threads() { return 1024; }

  private:
   cudaStream_t stream;
};

// The kernel objects the reference headers keep pointers to; the adapters leave them empty.
class CudaRecvPre {};
class CudaRecvPost {};

} // namespace PVCuda

namespace PV {

class PVParams;
class Communicator;

namespace Response {
enum Status { SUCCESS, NO_ACTION, PARTIAL, POSTPONE };
inline bool completed(Status s) { return s == SUCCESS or s == NO_ACTION; }
} // namespace Response

struct CommunicateInitInfoMessage {};
struct SetCudaDeviceMessage {
   PVCuda::CudaDevice *mCudaDevice;
};

class BaseObject {
  public:
   virtual ~BaseObject() {}
   void initialize(char const *name, PVParams *, Communicator const *) {
      mDescription = name ? name : "standin";
      setObjectType();
   }
   virtual void setObjectType() {}
   std::string const &getDescription() const { return mDescription; }
   char const *getDescription_c() const { return mDescription.c_str(); }
   std::string mObjectType;

  protected:
   std::string mDescription = "standin";
   bool mUsingGPUFlag              = false;
   PVCuda::CudaDevice *mCudaDevice = nullptr;

   friend struct Wiring;
};

// Shared weights: [arbor][kernel][nyp][nxp][nfp] in device memory.
class Weights {
  public:
   struct Geometry {
      std::vector<std::size_t> gSynPatchStart;
      std::vector<std::size_t> const &getGSynPatchStart() const { return gSynPatchStart; }
   };
   int nxp = 1, nyp = 1, nfp = 1, numDataPatches = 1;
   bool shared                    = true;
   PVCuda::CudaBuffer *deviceData = nullptr;
   std::shared_ptr<Geometry> geometry = std::make_shared<Geometry>();
   std::vector<Patch> patches;
   std::vector<float> hostData;

   bool getSharedFlag() const { return shared; }
   int getPatchSizeX() const { return nxp; }
   int getPatchSizeY() const { return nyp; }
   int getPatchSizeF() const { return nfp; }
   int getPatchSizeOverall() const { return nxp * nyp * nfp; }
   int getPatchStrideY() const { return nxp * nfp; }
   int getNumDataPatches() const { return numDataPatches; }
   void useGPU() {}
   void setCudaDevice(PVCuda::CudaDevice *) {}
   PVCuda::CudaBuffer *getDeviceData() const { return deviceData; }
   std::shared_ptr<Geometry> getGeometry() const { return geometry; }
   Patch const &getPatch(int k) const { return patches[k]; }
   float *getDataFromPatchIndex(int, int) { return hostData.data(); }
};

class WeightsPair {
  public:
   Weights *pre = nullptr, *post = nullptr;
   void needPre() {}
   void needPost() {}
   Weights *getPreWeights() { return pre; }
   Weights *getPostWeights() { return post; }
   bool getInitInfoCommunicatedFlag() const { return true; }
   bool getDataStructuresAllocatedFlag() const { return true; }
};

class ArborList {
  public:
   std::vector<int> delays{0};
   int getNumAxonalArbors() const { return (int)delays.size(); }
   int getDelay(int arbor) const { return delays[arbor]; }
};

class Publisher {
  public:
   PVLayerCube cube{};
   PVLayerCube createCube(int) const { return cube; }
};

// The presynaptic layer's published activity: the datastore, and for a sparse layer its
// SparseList, on the device; `updated` says the host copy is newer than the device's.
class BasePublisherComponent {
  public:
   PVLayerLoc loc{};
   bool sparse  = false;
   bool updated = false;
   Publisher publisher;
   PVCuda::CudaBuffer *datastore = nullptr, *activeIndices = nullptr, *numActive = nullptr;

   PVLayerLoc const *getLayerLoc() const { return &loc; }
   bool getSparseLayer() const { return sparse; }
   void setAllocCudaDatastore() {}
   void setAllocCudaActiveIndices() {}
   PVCuda::CudaBuffer *getCudaDatastore() { return datastore; }
   PVCuda::CudaBuffer *getCudaActiveIndices() { return activeIndices; }
   PVCuda::CudaBuffer *getCudaNumActive() { return numActive; }
   Publisher *getPublisher() { return &publisher; }
   bool getUpdatedCudaDatastoreFlag() const { return updated; }
   void setUpdatedCudaDatastoreFlag(bool f) { updated = f; }
};

class ComponentBuffer : public BaseObject {
  public:
   PVLayerLoc loc{};
   PVCuda::CudaBuffer *cudaBuffer = nullptr;
   PVLayerLoc const *getLayerLoc() const { return &loc; }
   int getBufferSize() const { return loc.nx * loc.ny * loc.nf; }
   int getBufferSizeAcrossBatch() const { return getBufferSize() * loc.nbatch; }
   PVCuda::CudaBuffer *getCudaBuffer() { return cudaBuffer; }
   void useCuda() {}
   bool getDataStructuresAllocatedFlag() const { return true; }
};

class LayerInputBuffer : public ComponentBuffer {};

class HyPerDelivery : public BaseObject {
  public:
   virtual void deliver(float *destBuffer)          = 0;
   virtual void deliverUnitInput(float *recvBuffer) = 0;
   ChannelType getChannelCode() const { return mChannelCode; }
   virtual Response::Status communicateInitInfo(std::shared_ptr<CommunicateInitInfoMessage const>) {
      return Response::SUCCESS;
   }
   virtual Response::Status setCudaDevice(std::shared_ptr<SetCudaDeviceMessage const> message) {
      mUsingGPUFlag = true;
      mCudaDevice   = message->mCudaDevice;
      return Response::SUCCESS;
   }
   virtual Response::Status allocateDataStructures() { return Response::SUCCESS; }
   virtual Response::Status copyInitialStateToGPU() { return Response::SUCCESS; }

  protected:
   bool mCorrectReceiveGpu                = false;
   bool mReceiveGpu                       = false;
   float mDeltaTimeFactor                 = 1.0f;
   ChannelType mChannelCode               = CHANNEL_EXC;
   BasePublisherComponent *mPreData = nullptr;
   LayerInputBuffer *mPostGSyn            = nullptr;
   WeightsPair *mWeightsPair              = nullptr;
   ArborList *mArborList                  = nullptr;

   friend struct Wiring;
};

} // namespace PV
