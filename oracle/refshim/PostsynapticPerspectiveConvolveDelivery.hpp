// PostsynapticPerspectiveConvolveDelivery.hpp -- stand-in declaration (same members as the reference class) so that the
// reference's delivery/PostsynapticPerspectiveConvolveDelivery.cpp compiles unmodified against refshim_delivery.hpp.
// It is force-included ahead of that file and defines the reference header's include guard,
// so the reference header is skipped.  TEST INFRASTRUCTURE ONLY.
#ifndef POSTSYNAPTICPERSPECTIVECONVOLVEDELIVERY_HPP_
#define POSTSYNAPTICPERSPECTIVECONVOLVEDELIVERY_HPP_
#include "refshim_delivery.hpp"

namespace PV {
class PostsynapticPerspectiveConvolveDelivery : public HyPerDelivery {
  public:
   PostsynapticPerspectiveConvolveDelivery(char const *name, PVParams *params, Communicator const *comm);
   PostsynapticPerspectiveConvolveDelivery();
   virtual ~PostsynapticPerspectiveConvolveDelivery();
   virtual void deliver(float *destBuffer) override;
   virtual void deliverUnitInput(float *recvBuffer) override;
   void initialize(char const *name, PVParams *params, Communicator const *comm);
   virtual void setObjectType() override;
   virtual Response::Status communicateInitInfo(std::shared_ptr<CommunicateInitInfoMessage const> message) override;
   virtual Response::Status allocateDataStructures() override;
};
}  // namespace PV
#endif
