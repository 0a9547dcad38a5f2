// Stand-in declaration of PV::PostsynapticPerspectiveGPUDelivery (the members of the
// reference's delivery/PostsynapticPerspectiveGPUDelivery.hpp, every method public).  TEST
// INFRASTRUCTURE ONLY.
#pragma once
#include "standin_framework.hpp"

namespace PV {
class PostsynapticPerspectiveGPUDelivery : public HyPerDelivery {
  public:
   PostsynapticPerspectiveGPUDelivery(char const *name, PVParams *params, Communicator const *comm);
   PostsynapticPerspectiveGPUDelivery();
   virtual ~PostsynapticPerspectiveGPUDelivery();
   virtual void deliver(float *destBuffer) override;
   virtual void deliverUnitInput(float *recvBuffer) override;
   void initialize(char const *name, PVParams *params, Communicator const *comm);
   virtual void setObjectType() override;
   virtual Response::Status communicateInitInfo(std::shared_ptr<CommunicateInitInfoMessage const> message) override;
   virtual Response::Status setCudaDevice(std::shared_ptr<SetCudaDeviceMessage const> message) override;
   virtual Response::Status allocateDataStructures() override;
   virtual Response::Status copyInitialStateToGPU() override;
   void initializeRecvKernelArgs();

   PVCuda::CudaRecvPost *mRecvKernel            = nullptr;
   PVCuda::CudaBuffer *mDevicePostToPreActivity = nullptr;
   PVCuda::CudaBuffer *mCudnnGSyn               = nullptr;
};
} // namespace PV
