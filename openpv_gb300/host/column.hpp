// column.hpp -- the host side of the LCA hot path as an OpenPV params file describes it, in
// C++ above the C ABI of libpvgpu.so.  It mirrors the reference's objects for this path:
//
//   HyPerCol            (columns/HyPerCol.cpp)         nx, ny, nbatch, dt; the phase loop
//   input layers        ImageLayer / PvpLayer           frames handed in by the host
//   HyPerLayer          V = G, A = V
//   ANNLayer            V = G, A = T(V)                 (components/ANNActivityBuffer.cpp)
//   ANNErrorLayer       V = errScale * G, A = T(V)      (ErrScaleInternalStateBuffer.cpp)
//   HyPerLCALayer       LCA update, A = T(V)            (HyPerLCAInternalStateBuffer.kpp)
//   MomentumLCALayer    LCA update with momentum        (MomentumLCAInternalStateBuffer.kpp)
//   ISTALayer           ISTA update                     (ISTAInternalStateBuffer.kpp)
//   LIFLayer            LIF update on channels EXC / INH / INHB (LIFActivityComponent.cpp)
//   HyPerConn / TransposeConn / IdentConn               (connections/*.cpp)
//
// and selects each connection's delivery by the keyword HyPerDeliveryCreator builds
// (delivery/HyPerDeliveryCreator.cpp:105-126) from receiveGpu, pvpatchAccumulateType and
// updateGSynFromPostPerspective.  Every delivery runs on the GPU: the "...GPUDelivery" keywords
// call the FAST kernels, the "...ConvolveDelivery" keywords (the reference's CPU path) call the
// REFERENCE_ORDER kernels, whose results are the reference CPU loops' bit for bit.  GSyn
// channels, the GSyn accumulator (channelCoefficients, default +1, -1) and sparse publication
// (sparseLayer: the SparseList built on the device) follow the reference components.
//
// Layer output (LayerOutputComponent.cpp): when the HyPerCol group names an outputPath, every
// layer with writeStep >= 0 (default dt) writes <outputPath>/<layer>.pvp -- sparse-values frames
// for sparse layers, packed on the device -- at initialWriteTime (default 0) and every writeStep
// after its phase publishes.  PvpLayer reads its frames from inputPath (.pvp) with the byFile
// batching of BatchIndexer (batch element b, display period d: frame (b + d * nbatch) mod F).
//
// Out of this drop-in (refused with a message): plasticity, delays, stochastic release, the
// adaptive time-scale probe, random initial V, layer types outside the list above.
#pragma once

#include "params.hpp"
#include "pvgpu.h"
#include "pvhost.h"

#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <string>
#include <vector>

namespace pvhost {

class Column;
struct Conn;

struct Layer {
   enum Kind { Input, HyPer, ANN, ANNError, LCA, MomentumLCA, ISTA, LIF } kind = HyPer;
   std::string name, keyword;
   int phase = 0;
   pvgpu_loc loc{};  // halo = the largest margin its outgoing connections need
   bool sparse = false;
   int numChannels = 0;
   std::vector<float> coeffs;  // GSynAccumulator channel coefficients
   // activity threshold (ANNActivityBuffer::applyVThresh / applyAMax)
   float VThresh = 0, AMin = 0, AMax = 0, AShift = 0, VWidth = 0;
   float errScale = 1.0f;                // ANNErrorLayer
   float tau = 1.0f;                     // HyPerLCALayer / MomentumLCALayer / ISTALayer timeConstantTau
   float momentumRate = 0.0f;            // MomentumLCALayer LCAMomentumRate
   bool selfInteract = true;             // HyPerLCALayer
   int displayPeriod = 0;                // input layers
   std::string inputPath;                // PvpLayer
   double initV = 0.0;                   // ConstantV initial state
   pvgpu_lif_params lif{};               // LIFLayer
   char lifMethod = 'a';
   double writeStep = -1.0, writeTime = 0.0;  // layer output
   pvhost_pvp_writer *out = nullptr;
   // device buffers
   float *gsyn = nullptr, *G = nullptr, *V = nullptr, *A = nullptr, *frames = nullptr, *prevDrive = nullptr;
   float *Vth = nullptr, *GE = nullptr, *GI = nullptr, *GIB = nullptr;  // LIF
   pvgpu_taus *rnd = nullptr;
   double *dtAdapt = nullptr;
   int numFrames = 0;
   pvgpu_entry *entries = nullptr;
   int64_t *numActive = nullptr;
   void *scratch = nullptr;
   size_t scratchBytes = 0;
   std::vector<Conn *> incoming;  // in params order

   int64_t numRes() const { return (int64_t)loc.nx * loc.ny * loc.nf; }
   int64_t numExt() const {
      return (int64_t)(loc.nx + loc.halo.lt + loc.halo.rt) * (loc.ny + loc.halo.dn + loc.halo.up) * loc.nf;
   }
};

// One HyPerDelivery subclass per reference keyword (same names).
class Delivery {
 public:
   explicit Delivery(Conn *c) : c_(c) {}
   virtual ~Delivery() = default;
   virtual const char *keyword() const = 0;
   // kernel family of the last deliver() (see pvhost_delivery_engine)
   virtual const char *engine() const { return engine_; }
   virtual pvgpu_status deliver(float *channel, cudaStream_t s) = 0;

 protected:
   Conn *c_;
   const char *engine_ = "none";
};

struct Conn {
   std::string name, keyword;
   Layer *pre = nullptr, *post = nullptr;
   int channel = 0;
   int nxp = 1, nyp = 1;
   bool receiveGpu = false, postPerspective = false;
   std::string accumulateType = "convolve";
   Conn *original = nullptr;  // TransposeConn
   std::vector<Conn *> transposes;
   float *W = nullptr;      // pre weights [kernel][nyp][nxp][nfp]
   float *Wpost = nullptr;  // post weights, when a post-perspective delivery needs them
   bool ownW = false, ownWpost = false;
   int64_t numWeights = 0;
   pvgpu_conn_desc desc{};
   std::unique_ptr<Delivery> delivery;
};

class Column {
 public:
   ~Column();
   // Builds the column from params text; false with a message on failure.
   bool build(const std::string &paramsText, std::string &err);
   pvgpu_status set_weights(const std::string &conn, const float *hostW, int64_t n, std::string &err);
   pvgpu_status set_input(const std::string &layer, const float *hostFrames, int numFrames, std::string &err);
   pvgpu_status set_state(const std::string &layer, const float *hostV, std::string &err);
   pvgpu_status advance(int numSteps, std::string &err);
   pvgpu_status read(const std::string &layer, int which, float *host, int64_t n, std::string &err);
   Layer *layer(const std::string &name);
   Conn *conn(const std::string &name);
   const std::vector<std::unique_ptr<Conn>> &conns() const { return conns_; }

 private:
   pvgpu_status step(std::string &err);
   pvgpu_status update(Layer &L, std::string &err);
   pvgpu_status output(Layer &L, double simTime, std::string &err);
   bool load_pvp_frames(Layer &L, std::string &err);
   pvgpu_status refresh_weights(Conn &c, std::string &err);
   bool allocate(std::string &err);

   Params params_;
   int nx_ = 0, ny_ = 0, nbatch_ = 1;
   double dt_ = 1.0;
   std::string outputPath_;
   uint32_t randomSeed_ = 1;
   bool initialOutputDone_ = false;
   int t_ = 0;
   int maxPhase_ = 0;
   cudaStream_t stream_ = nullptr;
   std::vector<std::unique_ptr<Layer>> layers_;
   std::vector<std::unique_ptr<Conn>> conns_;
   std::vector<void *> allocs_;
};

// The reference's Factory::createByKeyword for deliveries: nullptr for unknown keywords.
std::unique_ptr<Delivery> create_delivery(const std::string &keyword, Conn *c);

}  // namespace pvhost
