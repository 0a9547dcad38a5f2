// LIFActivityComponent.hpp -- stand-in declaration (same members as the reference class) so that the
// reference's components/LIFActivityComponent.cpp compiles unmodified into oracle/_ref.  It is
// force-included ahead of that file and defines the include guards of the reference headers the
// file names (its own header, checkpointing/CheckpointEntryRandState.hpp,
// components/InternalStateBuffer.hpp, observerpattern/ObserverTable.hpp), so those are skipped.
// The framework around the three update loops is reduced to what the file's other member
// functions need to compile; only the update loops are ever called.  TEST INFRASTRUCTURE ONLY.
#ifndef LIFACTIVITYCOMPONENT_HPP_
#define LIFACTIVITYCOMPONENT_HPP_
#define CHECKPOINTENTRYRANDSTATE_HPP_
#define INTERNALSTATEBUFFER_HPP_
#define OBSERVERTABLECOMPONENT_HPP_

#include "include/PVLayerLoc.h"
#include "include/default_params.h"
#include "include/pv_types.h"
#include "utils/PVAssert.hpp"
#include "utils/PVLog.hpp"
#include "utils/cl_random.h"
#include "utils/conversions.hpp"

#include <cerrno>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>

namespace PV {

enum ParamsIOFlag { PARAMS_IO_READ, PARAMS_IO_WRITE };

class PVParams {
  public:
   void ioParamValue(ParamsIOFlag, char const *, char const *, float *v, float dflt) { *v = dflt; }
   void ioParamString(ParamsIOFlag, char const *, char const *, char **v, char const *dflt, bool) {
      *v = strdup(dflt);
   }
};

class Communicator {
  public:
   int commRank() const { return 0; }
   int globalCommRank() const { return 0; }
   int communicator() const { return 0; }
};
inline int MPI_Barrier(int) { return 0; }

namespace Response {
enum Status { SUCCESS, NO_ACTION, PARTIAL, POSTPONE };
inline bool completed(Status s) { return s == SUCCESS || s == NO_ACTION; }
}  // namespace Response

struct ObjectTable {
   template <typename T>
   T *findObject(char const *) const { return nullptr; }
};
struct CommunicateInitInfoMessage {
   ObjectTable *mObjectTable = nullptr;
};
struct InitializeStateMessage {
   double mDeltaTime = 1.0;
};
class CheckpointEntryRandState {
  public:
   CheckpointEntryRandState(char const *, char const *, taus_uint4 *, PVLayerLoc const *, bool) {}
};
class Checkpointer {
  public:
   bool registerCheckpointEntry(std::shared_ptr<CheckpointEntryRandState>, bool) { return true; }
};
template <typename T>
struct RegisterDataMessage {
   T *mDataRegistry = nullptr;
};

class ComponentBuffer {
  public:
   ComponentBuffer(char const *name = "", PVParams * = nullptr, Communicator const * = nullptr) : mName(name) {}
   virtual ~ComponentBuffer() {}
   char const *getName() const { return mName.c_str(); }
   void setBufferLabel(char const *) {}
   float *getReadWritePointer() { return nullptr; }
   float const *getBufferData() const { return nullptr; }
   int getBufferSizeAcrossBatch() const { return 0; }
   template <typename M>
   void respond(M const &) {}
   static void checkDimensionsEqual(ComponentBuffer const *, ComponentBuffer const *) {}

  private:
   std::string mName;
};
class RestrictedBuffer : public ComponentBuffer {
   using ComponentBuffer::ComponentBuffer;
};
class InternalStateBuffer : public ComponentBuffer {
   using ComponentBuffer::ComponentBuffer;
};
class ActivityBuffer : public ComponentBuffer {
   using ComponentBuffer::ComponentBuffer;
};
class LayerInputBuffer : public ComponentBuffer {
  public:
   void requireChannel(int) {}
};

class Random {
  public:
   Random(PVLayerLoc const *, bool) {}
   taus_uint4 *getRNG(int) { return nullptr; }
};

class ActivityComponent {
  public:
   virtual ~ActivityComponent() {}

  protected:
   void initialize(char const *, PVParams *, Communicator const *) {}
   virtual void setObjectType() {}
   virtual void fillComponentTable() {}
   virtual int ioParamsFillGroup(ParamsIOFlag) { return 0; }
   virtual Response::Status communicateInitInfo(std::shared_ptr<CommunicateInitInfoMessage const>) {
      return Response::SUCCESS;
   }
   virtual Response::Status allocateDataStructures() { return Response::SUCCESS; }
   virtual Response::Status registerData(std::shared_ptr<RegisterDataMessage<Checkpointer> const>) {
      return Response::SUCCESS;
   }
   virtual Response::Status initializeState(std::shared_ptr<InitializeStateMessage const>) {
      return Response::SUCCESS;
   }
   virtual Response::Status updateActivity(double, double) { return Response::SUCCESS; }
   void addObserver(std::string const &, ComponentBuffer *) {}
   void addUniqueComponent(ComponentBuffer *) {}
   PVParams *parameters() const { return nullptr; }
   char const *getName() const { return name; }
   char const *getDescription_c() const { return name; }
   PVLayerLoc const *getLayerLoc() const { return nullptr; }

   char const *name = "LIF";
   std::string mObjectType;
   Communicator const *mCommunicator = nullptr;
   ActivityBuffer *mActivity = nullptr;
};

struct LIFParams {
   float Vrest = (float)V_REST;
   float Vexc = (float)V_EXC;
   float Vinh = (float)V_INH;
   float VinhB = (float)V_INHB;

   float VthRest = (float)VTH_REST;
   float tau = (float)TAU_VMEM;
   float tauVth = (float)TAU_VTH;
   float deltaVth = (float)DELTA_VTH;
   float deltaGIB = (float)DELTA_G_INHB;

   float noiseAmpE = 0.0f;
   float noiseAmpI = 0.0f;
   float noiseAmpIB = 0.0f;
   float noiseFreqE = 250.0f;
   float noiseFreqI = 250.0f;
   float noiseFreqIB = 250.0f;

   float tauE = (float)TAU_EXC;
   float tauI = (float)TAU_INH;
   float tauIB = (float)TAU_INHB;
};

class LIFActivityComponent : public ActivityComponent {
  protected:
   virtual void ioParam_Vrest(enum ParamsIOFlag ioFlag);
   virtual void ioParam_Vexc(enum ParamsIOFlag ioFlag);
   virtual void ioParam_Vinh(enum ParamsIOFlag ioFlag);
   virtual void ioParam_VinhB(enum ParamsIOFlag ioFlag);
   virtual void ioParam_tau(enum ParamsIOFlag ioFlag);
   virtual void ioParam_VthRest(enum ParamsIOFlag ioFlag);
   virtual void ioParam_tauVth(enum ParamsIOFlag ioFlag);
   virtual void ioParam_deltaVth(enum ParamsIOFlag ioFlag);
   virtual void ioParam_deltaGIB(enum ParamsIOFlag ioFlag);
   virtual void ioParam_noiseAmpE(enum ParamsIOFlag ioFlag);
   virtual void ioParam_noiseAmpI(enum ParamsIOFlag ioFlag);
   virtual void ioParam_noiseAmpIB(enum ParamsIOFlag ioFlag);
   virtual void ioParam_noiseFreqE(enum ParamsIOFlag ioFlag);
   virtual void ioParam_noiseFreqI(enum ParamsIOFlag ioFlag);
   virtual void ioParam_noiseFreqIB(enum ParamsIOFlag ioFlag);
   virtual void ioParam_tauE(enum ParamsIOFlag ioFlag);
   virtual void ioParam_tauI(enum ParamsIOFlag ioFlag);
   virtual void ioParam_tauIB(enum ParamsIOFlag ioFlag);
   virtual void ioParam_method(enum ParamsIOFlag ioFlag);

  public:
   LIFActivityComponent(char const *name, PVParams *params, Communicator const *comm);
   virtual ~LIFActivityComponent();

  protected:
   LIFActivityComponent() {}
   void initialize(char const *name, PVParams *params, Communicator const *comm);
   virtual void setObjectType() override;
   virtual void fillComponentTable() override;
   virtual RestrictedBuffer *createRestrictedBuffer(char const *label);
   virtual InternalStateBuffer *createInternalState();
   virtual int ioParamsFillGroup(enum ParamsIOFlag ioFlag) override;
   void checkMethodString();
   Response::Status communicateInitInfo(std::shared_ptr<CommunicateInitInfoMessage const> message) override;
   virtual Response::Status allocateDataStructures() override;
   virtual Response::Status registerData(std::shared_ptr<RegisterDataMessage<Checkpointer> const> message) override;
   void registerRandState(Checkpointer *checkpointer);
   virtual Response::Status initializeState(std::shared_ptr<InitializeStateMessage const> message) override;
   virtual Response::Status updateActivity(double simTime, double deltaTime) override;
   void updateActivityArma(int const nbatch, int const numNeurons, float const simTime, float const dt, int const nx,
                           int const ny, int const nf, int const lt, int const rt, int const dn, int const up,
                           LIFParams *params, taus_uint4 *rnd, float *V, float *Vth, float *G_E, float *G_I,
                           float *G_IB, float const *GSynHead, float *A);
   void updateActivityBeginning(int const nbatch, int const numNeurons, float const simTime, float const dt,
                                int const nx, int const ny, int const nf, int const lt, int const rt, int const dn,
                                int const up, LIFParams *params, taus_uint4 *rnd, float *V, float *Vth, float *G_E,
                                float *G_I, float *G_IB, float const *GSynHead, float *A);
   void updateActivityOriginal(int const nbatch, int const numNeurons, float const simTime, float const dt,
                               int const nx, int const ny, int const nf, int const lt, int const rt, int const dn,
                               int const up, LIFParams *params, taus_uint4 *rnd, float *V, float *Vth, float *G_E,
                               float *G_I, float *G_IB, float const *GSynHead, float *A);

   LIFParams mLIFParams;
   char *mMethodString = nullptr;
   char mMethod = 'a';
   RestrictedBuffer *mConductanceE = nullptr;
   RestrictedBuffer *mConductanceI = nullptr;
   RestrictedBuffer *mConductanceIB = nullptr;
   InternalStateBuffer *mInternalState = nullptr;
   LayerInputBuffer *mLayerInput = nullptr;
   Random *mRandState = nullptr;
   RestrictedBuffer *mVth = nullptr;
};

}  // namespace PV
#endif
