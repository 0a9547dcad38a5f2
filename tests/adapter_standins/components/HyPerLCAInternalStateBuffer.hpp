// Stand-in declaration of PV::HyPerLCAInternalStateBuffer: the members its GPU runKernel() reads
// (the reference's components/HyPerLCAInternalStateBuffer.hpp and HyPerInternalStateBuffer.hpp).
// TEST INFRASTRUCTURE ONLY.
#pragma once
#include "components/GSynAccumulator.hpp"

namespace PV {
class ActivityBuffer : public ComponentBuffer {};
class HyPerLCAInternalStateBuffer : public ComponentBuffer {
  public:
   void runKernel();
   double mScaledTimeConstantTau       = 1.0;
   bool mSelfInteract                  = true;
   GSynAccumulator *mAccumulatedGSyn   = nullptr;
   ActivityBuffer *mActivity           = nullptr;
   PVCuda::CudaBuffer *mCudaDtAdapt    = nullptr;
};
} // namespace PV
