// Stand-in declaration of PV::ANNActivityBuffer: the members its GPU runKernel() reads (the
// reference's components/ANNActivityBuffer.hpp and VInputActivityBuffer.hpp).  TEST
// INFRASTRUCTURE ONLY.
#pragma once
#include "standin_framework.hpp"

namespace PV {
class InternalStateBuffer : public ComponentBuffer {};
class ANNActivityBuffer : public ComponentBuffer {
  public:
   void runKernel();
   int mNumVertices                     = 0;
   PVCuda::CudaBuffer *mCudaVerticesV   = nullptr;
   PVCuda::CudaBuffer *mCudaVerticesA   = nullptr;
   PVCuda::CudaBuffer *mCudaSlopes      = nullptr;
   InternalStateBuffer *mInternalState  = nullptr;
};
} // namespace PV
