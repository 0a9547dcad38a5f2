// Stand-in declaration of PV::PresynapticPerspectiveGPUDelivery (the members of the reference's
// delivery/PresynapticPerspectiveGPUDelivery.hpp, every method public so that the test harness
// can run the framework's life cycle).  TEST INFRASTRUCTURE ONLY.
#pragma once
#include "standin_framework.hpp"

namespace PV {
class PresynapticPerspectiveGPUDelivery : public HyPerDelivery {
  public:
   PresynapticPerspectiveGPUDelivery(char const *name, PVParams *params, Communicator const *comm);
   PresynapticPerspectiveGPUDelivery();
   virtual ~PresynapticPerspectiveGPUDelivery();
   virtual void deliver(float *destBuffer) override;
   virtual void deliverUnitInput(float *recvBuffer) override;
   void initialize(char const *name, PVParams *params, Communicator const *comm);
   virtual void setObjectType() override;
   virtual Response::Status communicateInitInfo(std::shared_ptr<CommunicateInitInfoMessage const> message) override;
   virtual Response::Status setCudaDevice(std::shared_ptr<SetCudaDeviceMessage const> message) override;
   virtual Response::Status allocateDataStructures() override;
   virtual Response::Status copyInitialStateToGPU() override;
   void initializeRecvKernelArgs();

   PVCuda::CudaRecvPre *mRecvKernel          = nullptr;
   PVCuda::CudaBuffer *mDevicePatches        = nullptr;
   PVCuda::CudaBuffer *mDeviceGSynPatchStart = nullptr;
};
} // namespace PV
