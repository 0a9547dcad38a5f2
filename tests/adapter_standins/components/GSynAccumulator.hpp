// Stand-in declaration of PV::GSynAccumulator: the members its GPU runKernel() reads (the
// reference's components/GSynAccumulator.hpp).  TEST INFRASTRUCTURE ONLY.
#pragma once
#include "standin_framework.hpp"

namespace PV {
class GSynAccumulator : public ComponentBuffer {
  public:
   void runKernel();
   int mNumInputChannels = 0;
   std::vector<float> mChannelCoefficients;
   LayerInputBuffer *mLayerInput = nullptr;
};
} // namespace PV
