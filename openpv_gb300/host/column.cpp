// column.cpp -- see column.hpp.
#include "column.hpp"
#include "pvp.hpp"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <sstream>

namespace pvhost {

namespace {

// utils/requiredConvolveMargin.hpp, one axis
int required_margin(int nPre, int nPost, int patch) {
   if (nPre == nPost) return (patch - 1) / 2;
   if (nPre > nPost) return (patch - 1) * (nPre / nPost) / 2;
   return (patch / (nPost / nPre)) / 2;
}

// PatchSize::calcPostPatchSize (components/PatchSize.cpp:98-130), one axis
int post_patch_size(int prePatch, int nPre, int nPost) {
   if (nPre == nPost) return prePatch;
   if (nPre > nPost) return prePatch * (nPre / nPost);
   return prePatch / (nPost / nPre);
}

template <typename... Args>
std::string fmt(const Args &...args) {
   std::ostringstream o;
   (o << ... << args);
   return o.str();
}

// ---- the delivery classes (names and selection as in the reference) ------------------------

class PreDelivery : public Delivery {
 public:
   PreDelivery(Conn *c, int mode, const char *kw) : Delivery(c), mode_(mode), kw_(kw) {}
   const char *keyword() const override { return kw_; }
   pvgpu_status deliver(float *channel, cudaStream_t s) override {
      const Layer &pre = *c_->pre;
      engine_ = mode_ == PVGPU_DELIVER_FAST ? "simt" : "reference-order";
      if (pre.sparse)
         return pvgpu_deliver_pre(&c_->desc, pre.entries, pre.numActive, nullptr, c_->W, channel, mode_, s);
      return pvgpu_deliver_pre(&c_->desc, nullptr, nullptr, pre.A, c_->W, channel, mode_, s);
   }

 private:
   int mode_;
   const char *kw_;
};

// The GPU keyword tries the tensor-core form first (one-to-one connections with 32-multiple
// feature counts) and keeps the SIMT kernel for every other shape; the Convolve keyword always
// runs the reference-order kernel.
class PostDelivery : public Delivery {
 public:
   PostDelivery(Conn *c, int mode, const char *kw) : Delivery(c), mode_(mode), kw_(kw) {}
   ~PostDelivery() override {
      if (ws_) cudaFree(ws_);
   }
   const char *keyword() const override { return kw_; }
   pvgpu_status deliver(float *channel, cudaStream_t s) override {
      if (mode_ == PVGPU_DELIVER_FAST && tc_) {
         if (!ws_) {
            wsBytes_ = pvgpu_deliver_tc_workspace_bytes(&c_->desc);
            if (wsBytes_ == 0) {  // not a shape of the tensor-core entry
               tc_ = false;
               engine_ = "simt";
               return pvgpu_deliver_post(&c_->desc, c_->pre->A, c_->Wpost, channel, mode_, s);
            }
            if (cudaMalloc(&ws_, wsBytes_) != cudaSuccess) {
               ws_ = nullptr;
               return PVGPU_ERR_OOM;
            }
         }
         const pvgpu_status st = pvgpu_deliver_post_tc(&c_->desc, c_->pre->A, c_->Wpost, channel, ws_, wsBytes_, s);
         if (st != PVGPU_ERR_UNSUPPORTED_SHAPE) {
            engine_ = "tensor-core";
            return st;
         }
         tc_ = false;  // this geometry stays on the SIMT kernel
         cudaFree(ws_);
         ws_ = nullptr;
      }
      engine_ = mode_ == PVGPU_DELIVER_FAST ? "simt" : "reference-order";
      return pvgpu_deliver_post(&c_->desc, c_->pre->A, c_->Wpost, channel, mode_, s);
   }

 private:
   int mode_;
   const char *kw_;
   bool tc_ = true;
   void *ws_ = nullptr;
   size_t wsBytes_ = 0;
};

class IdentDeliveryImpl : public Delivery {
 public:
   using Delivery::Delivery;
   const char *keyword() const override { return "IdentDelivery"; }
   pvgpu_status deliver(float *channel, cudaStream_t s) override {
      const Layer &pre = *c_->pre;
      engine_ = "ident";
      return pvgpu_deliver_ident(&c_->desc.pre, &c_->desc.post, pre.sparse ? pre.entries : nullptr,
                                 pre.sparse ? pre.numActive : nullptr, pre.sparse ? nullptr : pre.A, channel, s);
   }
};

}  // namespace

std::unique_ptr<Delivery> create_delivery(const std::string &kw, Conn *c) {
   if (kw == "PresynapticPerspectiveGPUDelivery")
      return std::make_unique<PreDelivery>(c, PVGPU_DELIVER_FAST, "PresynapticPerspectiveGPUDelivery");
   if (kw == "PresynapticPerspectiveConvolveDelivery")
      return std::make_unique<PreDelivery>(c, PVGPU_DELIVER_REFERENCE_ORDER, "PresynapticPerspectiveConvolveDelivery");
   if (kw == "PostsynapticPerspectiveGPUDelivery")
      return std::make_unique<PostDelivery>(c, PVGPU_DELIVER_FAST, "PostsynapticPerspectiveGPUDelivery");
   if (kw == "PostsynapticPerspectiveConvolveDelivery")
      return std::make_unique<PostDelivery>(c, PVGPU_DELIVER_REFERENCE_ORDER,
                                            "PostsynapticPerspectiveConvolveDelivery");
   if (kw == "IdentDelivery") return std::make_unique<IdentDeliveryImpl>(c);
   return nullptr;
}

// ---- column ---------------------------------------------------------------------------------

Column::~Column() {
   if (stream_) cudaStreamSynchronize(stream_);
   for (auto &L : layers_)
      if (L->out) pvhost_pvp_writer_close(L->out);
   for (void *p : allocs_) cudaFree(p);
   if (stream_) cudaStreamDestroy(stream_);
}

Layer *Column::layer(const std::string &name) {
   for (auto &l : layers_)
      if (l->name == name) return l.get();
   return nullptr;
}

Conn *Column::conn(const std::string &name) {
   for (auto &c : conns_)
      if (c->name == name) return c.get();
   return nullptr;
}

bool Column::build(const std::string &text, std::string &err) {
   if (!parse_params(text, params_, err)) return false;
   const ParamGroup *col = nullptr;
   for (const auto &g : params_.groups)
      if (g.keyword == "HyPerCol") col = &g;
   if (!col) {
      err = "params: no HyPerCol group";
      return false;
   }
   nx_ = (int)col->number("nx", 0);
   ny_ = (int)col->number("ny", 0);
   nbatch_ = (int)col->number("nbatch", 1);
   dt_ = col->number("dt", 1.0);
   outputPath_ = col->string("outputPath", "");
   randomSeed_ = (uint32_t)col->number("randomSeed", 1.0);
   if (nx_ <= 0 || ny_ <= 0 || nbatch_ <= 0 || dt_ <= 0) {
      err = fmt("HyPerCol \"", col->name, "\": nx, ny, nbatch and dt must be positive");
      return false;
   }
   // layers
   for (const auto &g : params_.groups) {
      static const std::map<std::string, Layer::Kind> kinds = {
            {"ImageLayer", Layer::Input}, {"PvpLayer", Layer::Input},     {"HyPerLayer", Layer::HyPer},
            {"ANNLayer", Layer::ANN},     {"ANNErrorLayer", Layer::ANNError}, {"HyPerLCALayer", Layer::LCA},
            {"MomentumLCALayer", Layer::MomentumLCA}, {"ISTALayer", Layer::ISTA}, {"LIFLayer", Layer::LIF}};
      auto k = kinds.find(g.keyword);
      if (k == kinds.end()) {
         if (g.keyword.size() > 5 && g.keyword.compare(g.keyword.size() - 5, 5, "Layer") == 0) {
            err = fmt("layer type ", g.keyword, " is outside this drop-in (inputs, HyPerLayer, ANNLayer, "
                                                "ANNErrorLayer, HyPerLCALayer, MomentumLCALayer, ISTALayer, LIFLayer)");
            return false;
         }
         continue;
      }
      auto L = std::make_unique<Layer>();
      L->kind = k->second;
      L->name = g.name;
      L->keyword = g.keyword;
      L->phase = (int)g.number("phase", 0);
      L->sparse = g.flag("sparseLayer", false);
      const double sx = g.number("nxScale", 1.0), sy = g.number("nyScale", 1.0);
      L->loc.nbatch = nbatch_;
      L->loc.nx = (int)std::lround(sx * nx_);
      L->loc.ny = (int)std::lround(sy * ny_);
      L->loc.nf = (int)g.number("nf", 1);
      if (L->loc.nx <= 0 || L->loc.ny <= 0 || L->loc.nf <= 0) {
         err = fmt("layer \"", g.name, "\": empty size");
         return false;
      }
      // ANNActivityBuffer parameters (components/ANNActivityBuffer.cpp:135-165, defaults
      // VThresh = -FLT_MAX, AMin = VThresh, AMax = FLT_MAX, AShift = 0, VWidth = 0)
      L->VThresh = (float)g.number("VThresh", -FLT_MAX);
      L->AMin = (float)g.number("AMin", L->VThresh);
      L->AMax = (float)g.number("AMax", FLT_MAX);
      L->AShift = (float)g.number("AShift", 0.0);
      L->VWidth = (float)g.number("VWidth", 0.0);
      if (L->VWidth < 0) {  // ANNActivityBuffer: a negative width moves the threshold down
         L->VThresh += L->VWidth;
         L->VWidth = -L->VWidth;
      }
      if (L->kind == Layer::HyPer) {
         L->VThresh = -FLT_MAX;
         L->AMin = -FLT_MAX;
         L->AMax = FLT_MAX;
         L->AShift = 0;
         L->VWidth = 0;
      }
      if (g.has("verticesV") || g.has("verticesA")) {
         err = fmt("layer \"", g.name, "\": piecewise-linear vertices are outside this drop-in");
         return false;
      }
      L->errScale = (float)g.number("errScale", 1.0);
      L->tau = (float)g.number("timeConstantTau", 1.0);
      L->momentumRate = (float)g.number("LCAMomentumRate", 0.0);
      L->selfInteract = g.flag("selfInteract", true);
      L->displayPeriod = (int)g.number("displayPeriod", 0);
      L->inputPath = g.string("inputPath", "");
      // LayerOutputComponent: writeStep defaults to dt when absent, initialWriteTime to 0
      L->writeStep = g.number("writeStep", dt_);
      L->writeTime = g.number("initialWriteTime", 0.0);
      if (L->kind == Layer::LIF) {
         // LIFParams (components/LIFActivityComponent.hpp:22-45) with default_params.h defaults
         pvgpu_lif_params &q = L->lif;
         q.Vrest = (float)g.number("Vrest", -70.0);
         q.Vexc = (float)g.number("Vexc", 0.0);
         q.Vinh = (float)g.number("Vinh", -75.0);
         q.VinhB = (float)g.number("VinhB", -90.0);
         q.VthRest = (float)g.number("VthRest", -55.0);
         q.tau = (float)g.number("tau", 20.0);
         q.tauVth = (float)g.number("tauVth", 10.0);
         q.deltaVth = (float)g.number("deltaVth", 5.0);
         q.deltaGIB = (float)g.number("deltaGIB", 1.0);
         q.noiseAmpE = (float)g.number("noiseAmpE", 0.0);
         q.noiseAmpI = (float)g.number("noiseAmpI", 0.0);
         q.noiseAmpIB = (float)g.number("noiseAmpIB", 0.0);
         // noise frequencies are capped at one event per step (LIFActivityComponent::initializeState)
         const float maxFreq = (float)(1000.0 / dt_);
         q.noiseFreqE = std::min((float)g.number("noiseFreqE", 250.0), maxFreq);
         q.noiseFreqI = std::min((float)g.number("noiseFreqI", 250.0), maxFreq);
         q.noiseFreqIB = std::min((float)g.number("noiseFreqIB", 250.0), maxFreq);
         q.tauE = (float)g.number("tauE", 1.0);
         q.tauI = (float)g.number("tauI", 5.0);
         q.tauIB = (float)g.number("tauIB", 10.0);
         const std::string method = g.string("method", "arma");
         L->lifMethod = method.empty() ? 'a' : method[0];
         if (L->lifMethod != 'a' && L->lifMethod != 'b' && L->lifMethod != 'o') {
            err = fmt("layer \"", g.name, "\": method \"", method, "\" (arma, beginning or original)");
            return false;
         }
         L->numChannels = 3;  // EXC, INH, INHB
      }
      if (g.has("adaptiveTimeScaleProbe") && !g.string("adaptiveTimeScaleProbe", "").empty()) {
         err = fmt("layer \"", g.name, "\": the adaptive time-scale probe is outside this drop-in (fixed dt)");
         return false;
      }
      const std::string initV = g.string("InitVType", "ZeroV");
      if (initV == "ConstantV") L->initV = g.number("valueV", 0.0);
      else if (initV != "ZeroV") {
         err = fmt("layer \"", g.name, "\": InitVType ", initV + " is outside this drop-in (ZeroV, ConstantV; or "
                                                               "set the state through the API)");
         return false;
      }
      // GSynAccumulator coefficients (components/GSynAccumulator.cpp: default {+1, -1})
      L->coeffs = {1.0f, -1.0f};
      const ParamValue *ci = g.find("channelIndices"), *cc = g.find("channelCoefficients");
      if (ci || cc) {
         if (!ci || !cc || ci->array.size() != cc->array.size()) {
            err = fmt("layer \"", g.name, "\": channelIndices and channelCoefficients differ in length");
            return false;
         }
         for (size_t i = 0; i < ci->array.size(); i++) {
            const int ch = (int)ci->array[i];
            if (ch < 0) continue;
            if (ch >= (int)L->coeffs.size()) L->coeffs.resize(ch + 1, 0.0f);
            L->coeffs[ch] = (float)cc->array[i];
         }
      }
      maxPhase_ = std::max(maxPhase_, L->phase);
      layers_.push_back(std::move(L));
   }
   // connections
   for (const auto &g : params_.groups) {
      if (g.keyword != "HyPerConn" && g.keyword != "TransposeConn" && g.keyword != "IdentConn") {
         if (g.keyword.size() > 4 && g.keyword.compare(g.keyword.size() - 4, 4, "Conn") == 0) {
            err = fmt("connection type ", g.keyword, " is outside this drop-in (HyPerConn, TransposeConn, IdentConn)");
            return false;
         }
         continue;
      }
      auto c = std::make_unique<Conn>();
      c->name = g.name;
      c->keyword = g.keyword;
      c->pre = layer(g.string("preLayerName", ""));
      c->post = layer(g.string("postLayerName", ""));
      if (!c->pre || !c->post) {
         err = fmt("connection \"", g.name, "\": unknown preLayerName or postLayerName");
         return false;
      }
      c->channel = (int)g.number("channelCode", 0);
      if (c->channel < 0 || c->channel > 3) {
         err = fmt("connection \"", g.name, "\": channelCode outside 0..3");
         return false;
      }
      if (g.flag("plasticityFlag", false) || g.number("delay", 0.0) != 0.0 || !g.flag("sharedWeights", true) ||
          g.flag("convertRateToSpikeCount", false)) {
         err = fmt("connection \"", g.name, "\": plasticity, delays, non-shared weights and rate conversion are "
                                            "outside this drop-in");
         return false;
      }
      c->receiveGpu = g.flag("receiveGpu", false);
      c->postPerspective = g.flag("updateGSynFromPostPerspective", false);
      c->accumulateType = g.string("pvpatchAccumulateType", "convolve");
      const Layer &pre = *c->pre, &post = *c->post;
      if (g.keyword == "IdentConn") {
         c->nxp = c->nyp = 1;
      } else if (g.keyword == "TransposeConn") {
         c->original = conn(g.string("originalConnName", ""));
         if (!c->original || c->original->keyword != "HyPerConn" || c->original->pre != c->post ||
             c->original->post != c->pre) {
            err = fmt("TransposeConn \"", g.name, "\": originalConnName must name an earlier HyPerConn from this "
                                                  "connection's post layer to its pre layer");
            return false;
         }
         c->original->transposes.push_back(c.get());
         // the transpose's patch is the original's post-patch size (TransposeConn / PatchSize)
         c->nxp = post_patch_size(c->original->nxp, post.loc.nx, pre.loc.nx);
         c->nyp = post_patch_size(c->original->nyp, post.loc.ny, pre.loc.ny);
      } else {
         c->nxp = (int)g.number("nxp", 1);
         c->nyp = (int)g.number("nyp", c->nxp);
         const int nfp = (int)g.number("nfp", post.loc.nf);
         if (nfp != post.loc.nf) {
            err = fmt("connection \"", g.name, "\": nfp differs from the post layer's nf");
            return false;
         }
      }
      // HyPerDeliveryCreator::create: "{Pre,Post}synapticPerspective{GPU,Convolve,Stochastic}Delivery"
      std::string kw;
      if (g.keyword == "IdentConn") {
         kw = "IdentDelivery";
      } else {
         const char *type = c->receiveGpu ? "GPU" : c->accumulateType == "convolve" ? "Convolve"
                                                  : c->accumulateType == "stochastic" ? "Stochastic"
                                                                                      : "";
         if (!*type) {
            err = fmt("connection \"", g.name, "\": pvpatchAccumulateType \"", c->accumulateType + "\" is unrecognized");
            return false;
         }
         kw = std::string(c->postPerspective ? "Post" : "Pre") + "synapticPerspective" + type + "Delivery";
      }
      c->delivery = create_delivery(kw, c.get());
      if (!c->delivery) {
         err = fmt("connection \"", g.name, "\": delivery ", kw + " is outside this drop-in");
         return false;
      }
      c->post->incoming.push_back(c.get());
      conns_.push_back(std::move(c));
   }
   // margins: each layer's halo is the largest margin its outgoing connections require
   // (requiredConvolveMargin, as HyPerConn's communicateInitInfo requests of the pre layer)
   for (auto &c : conns_) {
      Layer &pre = *c->pre;
      const Layer &post = *c->post;
      const int mx = c->keyword == "IdentConn" ? 0 : required_margin(pre.loc.nx, post.loc.nx, c->nxp);
      const int my = c->keyword == "IdentConn" ? 0 : required_margin(pre.loc.ny, post.loc.ny, c->nyp);
      const int m = std::max(mx, my);
      if (m > pre.loc.halo.lt) pre.loc.halo = {m, m, m, m};
   }
   for (auto &c : conns_) {
      c->desc.pre = c->pre->loc;
      c->desc.post = c->post->loc;
      c->desc.nxp = c->nxp;
      c->desc.nyp = c->nyp;
      c->desc.dt_factor = 1.0f;
      const int64_t nk = (int64_t)(c->pre->loc.nx > c->post->loc.nx ? c->pre->loc.nx / c->post->loc.nx : 1) *
                         (c->pre->loc.ny > c->post->loc.ny ? c->pre->loc.ny / c->post->loc.ny : 1) * c->pre->loc.nf;
      c->numWeights = nk * c->nxp * c->nyp * c->post->loc.nf;
      Layer &post = *c->post;
      post.numChannels = std::max(post.numChannels, c->channel + 1);
   }
   return allocate(err);
}

bool Column::allocate(std::string &err) {
   if (cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking) != cudaSuccess) {
      err = "cudaStreamCreate failed";
      return false;
   }
   auto dalloc = [&](size_t bytes) -> void * {
      void *p = nullptr;
      if (bytes == 0) bytes = 4;
      if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
      cudaMemsetAsync(p, 0, bytes, stream_);
      allocs_.push_back(p);
      return p;
   };
   for (auto &L : layers_) {
      const size_t nb = (size_t)nbatch_;
      L->A = (float *)dalloc(L->numExt() * nb * 4);
      if (L->kind != Layer::Input) {
         L->numChannels = std::max(L->numChannels, 1);
         L->gsyn = (float *)dalloc(L->numRes() * nb * L->numChannels * 4);
         L->G = (float *)dalloc(L->numRes() * nb * 4);
         const bool ownV = L->kind == Layer::LCA || L->kind == Layer::MomentumLCA || L->kind == Layer::ISTA;
         L->V = ownV ? (float *)dalloc(L->numRes() * nb * 4) : L->G;
         if (L->kind == Layer::MomentumLCA) {
            L->prevDrive = (float *)dalloc(L->numRes() * nb * 4);
            if (!L->prevDrive) break;
         }
         if (L->kind == Layer::LIF) {
            L->V = (float *)dalloc(L->numRes() * nb * 4);
            L->Vth = (float *)dalloc(L->numRes() * nb * 4);
            L->GE = (float *)dalloc(L->numRes() * nb * 4);
            L->GI = (float *)dalloc(L->numRes() * nb * 4);
            L->GIB = (float *)dalloc(L->numRes() * nb * 4);
            L->rnd = (pvgpu_taus *)dalloc(L->numRes() * nb * sizeof(pvgpu_taus));
            if (!L->V || !L->Vth || !L->GE || !L->GI || !L->GIB || !L->rnd) break;
         }
         L->dtAdapt = (double *)dalloc(nb * sizeof(double));
         if (!L->A || !L->gsyn || !L->G || !L->V || !L->dtAdapt) break;
         std::vector<double> dts(nb, dt_);
         cudaMemcpyAsync(L->dtAdapt, dts.data(), nb * sizeof(double), cudaMemcpyHostToDevice, stream_);
         cudaStreamSynchronize(stream_);
      }
      if (L->sparse) {
         L->entries = (pvgpu_entry *)dalloc(L->numExt() * nb * sizeof(pvgpu_entry));
         L->numActive = (int64_t *)dalloc(nb * sizeof(int64_t));
         L->scratchBytes = pvgpu_compact_scratch_bytes(nbatch_, L->numExt());
         L->scratch = dalloc(L->scratchBytes);
         if (!L->entries || !L->numActive || !L->scratch) break;
      }
   }
   for (auto &L : layers_) {
      if (!L->A || (L->kind != Layer::Input && (!L->gsyn || !L->G || !L->V)) || (L->sparse && !L->scratch)) {
         err = "device allocation failed";
         return false;
      }
   }
   // initial state: V from InitVType, A = T(V), published (HyPerActivityBuffer::initializeState)
   for (auto &L : layers_) {
      if (L->kind == Layer::Input) continue;
      if (L->kind == Layer::LIF) {
         // LIFActivityComponent::initializeState: conductances 0, Vth = VthRest; V from InitVType;
         // generator states seeded from the column's randomSeed (cl_random_init layout); A = 0
         const size_t n = (size_t)L->numRes() * nbatch_;
         std::vector<float> v(n, (float)L->initV), vth(n, L->lif.VthRest);
         pvgpu_status s = pvgpu_taus_init(L->rnd, (int64_t)n, randomSeed_, stream_);
         if (s != PVGPU_OK || cudaMemcpyAsync(L->V, v.data(), n * 4, cudaMemcpyHostToDevice, stream_) != cudaSuccess ||
             cudaMemcpyAsync(L->Vth, vth.data(), n * 4, cudaMemcpyHostToDevice, stream_) != cudaSuccess ||
             cudaStreamSynchronize(stream_) != cudaSuccess) {
            err = "LIF initial state failed";
            return false;
         }
         if (L->sparse &&
             pvgpu_compact_active(L->A, nbatch_, L->numExt(), L->entries, L->numActive, L->scratch, L->scratchBytes,
                                  stream_) != PVGPU_OK) {
            err = std::string("initial state: ") + pvgpu_last_error();
            return false;
         }
         continue;
      }
      if (L->initV != 0.0) {
         std::vector<float> v((size_t)L->numRes() * nbatch_, (float)L->initV);
         std::string e2;
         if (set_state(L->name, v.data(), e2) != PVGPU_OK) {
            err = e2;
            return false;
         }
      } else {
         cudaMemsetAsync(L->V, 0, L->numRes() * nbatch_ * 4, stream_);
         pvgpu_status s = pvgpu_ann_activity(&L->loc, L->V, L->VThresh, L->AMin, L->AMax, L->AShift, L->VWidth, L->A,
                                             stream_);
         if (s == PVGPU_OK && L->sparse)
            s = pvgpu_compact_active(L->A, nbatch_, L->numExt(), L->entries, L->numActive, L->scratch, L->scratchBytes,
                                     stream_);
         if (s != PVGPU_OK) {
            err = std::string("initial state: ") + pvgpu_last_error();
            return false;
         }
      }
   }
   if (cudaStreamSynchronize(stream_) != cudaSuccess) {
      err = "initialisation failed on the device";
      return false;
   }
   for (auto &L : layers_) {
      if (L->keyword == "PvpLayer" && !L->inputPath.empty() && !load_pvp_frames(*L, err)) return false;
      if (!outputPath_.empty() && L->writeStep >= 0) {
         const std::string path = outputPath_ + "/" + L->name + ".pvp";
         if (pvhost_pvp_writer_open(path.c_str(), L->loc.nx, L->loc.ny, L->loc.nf, L->sparse ? 1 : 0, &L->out) !=
             PVGPU_OK) {
            err = fmt("layer \"", L->name, "\": ") + pvhost_last_error();
            return false;
         }
      }
   }
   return true;
}

// PvpLayer frames (InputActivityBuffer with batchMethod byFile, components/BatchIndexer.cpp:60-83):
// batch element b in display period d shows file frame (b + d * nbatch) mod F; the frame sequence
// repeats after F / gcd(F, nbatch) display periods, which are loaded here.
bool Column::load_pvp_frames(Layer &L, std::string &err) {
   PvpReader r;
   if (!r.open(L.inputPath, err)) return false;
   const PvpHeader &h = r.header();
   if (h.nx != L.loc.nx || h.ny != L.loc.ny || h.nf != L.loc.nf || r.num_frames() <= 0) {
      err = fmt("layer \"", L.name, "\": ", L.inputPath, " holds ", h.nx, "x", h.ny, "x", h.nf, " frames (",
                r.num_frames(), ")");
      return false;
   }
   const int F = r.num_frames();
   int a = F, b = nbatch_;
   while (b) {
      const int t = a % b;
      a = b;
      b = t;
   }
   const int D = F / a;
   const size_t n = (size_t)L.numRes();
   std::vector<float> frames((size_t)D * nbatch_ * n);
   for (int d = 0; d < D; d++)
      for (int bb = 0; bb < nbatch_; bb++)
         if (!r.read_dense((bb + d * nbatch_) % F, frames.data() + ((size_t)d * nbatch_ + bb) * n, nullptr, err))
            return false;
   return set_input(L.name, frames.data(), D, err) == PVGPU_OK;
}

// LayerOutputComponent::outputState (components/LayerOutputComponent.cpp:183-197).
pvgpu_status Column::output(Layer &L, double simTime, std::string &err) {
   if (!L.out || L.writeStep < 0 || simTime < L.writeTime - dt_ / 2) return PVGPU_OK;
   L.writeTime += L.writeStep;
   pvgpu_status s = L.sparse ? pvhost_pvp_write_sparse_device(L.out, &L.loc, L.entries, L.numActive, simTime, stream_)
                             : pvhost_pvp_write_dense_device(L.out, &L.loc, L.A, simTime, stream_);
   if (s != PVGPU_OK) err = fmt("layer \"", L.name, "\" output: ") + pvhost_last_error();
   return s;
}

pvgpu_status Column::refresh_weights(Conn &c, std::string &err) {
   // post weights for a post-perspective HyPerConn; pre weights of its transposes
   auto need = [&](float *&buf, bool &own) -> bool {
      if (buf && own) return true;
      void *p = nullptr;
      if (cudaMalloc(&p, c.numWeights * 4) != cudaSuccess) return false;
      allocs_.push_back(p);
      buf = (float *)p;
      own = true;
      return true;
   };
   if (c.postPerspective) {
      if (!need(c.Wpost, c.ownWpost)) return PVGPU_ERR_OOM;
      pvgpu_status s = pvgpu_transpose_weights(&c.desc, c.W, c.Wpost, stream_);
      if (s != PVGPU_OK) return s;
   }
   for (Conn *t : c.transposes) {
      // the transpose's post weights are the original's pre weights; its pre weights are the
      // original's post weights
      t->Wpost = c.W;
      t->ownWpost = false;
      t->numWeights = c.numWeights;
      if (!t->postPerspective) {
         if (!need(t->W, t->ownW)) return PVGPU_ERR_OOM;
         pvgpu_status s = pvgpu_transpose_weights(&c.desc, c.W, t->W, stream_);
         if (s != PVGPU_OK) return s;
      }
   }
   (void)err;
   return PVGPU_OK;
}

pvgpu_status Column::set_weights(const std::string &name, const float *hostW, int64_t n, std::string &err) {
   Conn *c = conn(name);
   if (!c || c->keyword != "HyPerConn") {
      err = fmt("set_weights: \"", name, "\" is not a HyPerConn of the column");
      return PVGPU_ERR_BAD_ARG;
   }
   if (n != c->numWeights || !hostW) {
      std::ostringstream o;
      o << "set_weights: \"" << name << "\" takes " << c->numWeights << " weights ([kernel][nyp][nxp][nfp])";
      err = o.str();
      return PVGPU_ERR_BAD_ARG;
   }
   if (!c->W) {
      void *p = nullptr;
      if (cudaMalloc(&p, n * 4) != cudaSuccess) return PVGPU_ERR_OOM;
      allocs_.push_back(p);
      c->W = (float *)p;
      c->ownW = true;
   }
   if (cudaMemcpyAsync(c->W, hostW, n * 4, cudaMemcpyHostToDevice, stream_) != cudaSuccess) return PVGPU_ERR_LAUNCH;
   pvgpu_status s = refresh_weights(*c, err);
   if (s == PVGPU_OK && cudaStreamSynchronize(stream_) != cudaSuccess) s = PVGPU_ERR_LAUNCH;
   return s;
}

pvgpu_status Column::set_input(const std::string &name, const float *hostFrames, int numFrames, std::string &err) {
   Layer *L = layer(name);
   if (!L || L->kind != Layer::Input || numFrames <= 0 || !hostFrames) {
      err = fmt("set_input: \"", name, "\" is not an input layer of the column (or no frames)");
      return PVGPU_ERR_BAD_ARG;
   }
   const size_t bytes = (size_t)numFrames * nbatch_ * L->numRes() * 4;
   if (L->frames) cudaFree(L->frames);
   allocs_.erase(std::remove(allocs_.begin(), allocs_.end(), (void *)L->frames), allocs_.end());
   void *p = nullptr;
   if (cudaMalloc(&p, bytes) != cudaSuccess) return PVGPU_ERR_OOM;
   L->frames = (float *)p;
   allocs_.push_back(p);
   L->numFrames = numFrames;
   if (cudaMemcpyAsync(L->frames, hostFrames, bytes, cudaMemcpyHostToDevice, stream_) != cudaSuccess ||
       cudaStreamSynchronize(stream_) != cudaSuccess)
      return PVGPU_ERR_LAUNCH;
   return PVGPU_OK;
}

pvgpu_status Column::set_state(const std::string &name, const float *hostV, std::string &err) {
   Layer *L = layer(name);
   if (!L || L->kind == Layer::Input || !hostV) {
      err = fmt("set_state: \"", name, "\" is not a non-input layer of the column");
      return PVGPU_ERR_BAD_ARG;
   }
   const size_t n = (size_t)L->numRes() * nbatch_;
   if (cudaMemcpyAsync(L->V, hostV, n * 4, cudaMemcpyHostToDevice, stream_) != cudaSuccess) return PVGPU_ERR_LAUNCH;
   // A = T(V), published (HyPerActivityBuffer::initializeState)
   pvgpu_status s = pvgpu_ann_activity(&L->loc, L->V, L->VThresh, L->AMin, L->AMax, L->AShift, L->VWidth, L->A, stream_);
   if (s == PVGPU_OK && L->sparse)
      s = pvgpu_compact_active(L->A, nbatch_, L->numExt(), L->entries, L->numActive, L->scratch, L->scratchBytes,
                               stream_);
   if (s == PVGPU_OK && cudaStreamSynchronize(stream_) != cudaSuccess) s = PVGPU_ERR_LAUNCH;
   return s;
}

// One layer's update after its deliveries: G = sum c_ch GSyn[ch]; V per the layer type;
// A = T(V) into the extended buffer (halo stays zero); SparseList when sparseLayer.
pvgpu_status Column::update(Layer &L, std::string &err) {
   const int64_t n = L.numRes() * nbatch_;
   pvgpu_status s = PVGPU_OK;
   if (L.kind == Layer::Input) {
      if (!L.frames) {
         err = fmt("input layer \"", L.name, "\" has no frames (set_input)");
         return PVGPU_ERR_BAD_ARG;
      }
      // InputLayer: frame (t-1) / displayPeriod, cycling; the restricted frame into A
      const int frame = L.displayPeriod > 0 ? ((t_ - 1) / L.displayPeriod) % L.numFrames : 0;
      const float *src = L.frames + (size_t)frame * n;
      s = pvgpu_ann_activity(&L.loc, src, -FLT_MAX, -FLT_MAX, FLT_MAX, 0.0f, 0.0f, L.A, stream_);
   } else if (L.kind == Layer::LIF) {
      // the three channels as LIFActivityComponent reads them (GSynHead, channel-major)
      s = pvgpu_lif_update(&L.loc, L.lifMethod, &L.lif, (float)dt_, L.rnd, L.V, L.Vth, L.GE, L.GI, L.GIB, L.gsyn, L.A,
                           stream_);
   } else {
      const int nch = std::min(L.numChannels, (int)L.coeffs.size());
      s = pvgpu_gsyn_accumulate(n, nch, L.coeffs.data(), L.gsyn, L.G, stream_);
      if (s == PVGPU_OK && L.kind == Layer::ANNError && L.errScale != 1.0f) s = pvgpu_err_scale(n, L.errScale, L.V, stream_);
      if (s == PVGPU_OK && L.kind == Layer::LCA)
         s = pvgpu_lca_update(&L.loc, L.selfInteract ? 1 : 0, L.dtAdapt, (float)(L.tau / dt_), L.G, L.A, L.V, stream_);
      if (s == PVGPU_OK && L.kind == Layer::MomentumLCA)
         s = pvgpu_momentum_lca_update(&L.loc, L.selfInteract ? 1 : 0, L.momentumRate, L.dtAdapt, (float)(L.tau / dt_),
                                       L.G, L.A, L.prevDrive, L.V, stream_);
      if (s == PVGPU_OK && L.kind == Layer::ISTA)
         s = pvgpu_ista_update(&L.loc, L.VThresh, L.dtAdapt, (float)(L.tau / dt_), L.G, L.A, L.V, stream_);
      if (s == PVGPU_OK)
         s = pvgpu_ann_activity(&L.loc, L.V, L.VThresh, L.AMin, L.AMax, L.AShift, L.VWidth, L.A, stream_);
   }
   if (s == PVGPU_OK && L.sparse)
      s = pvgpu_compact_active(L.A, nbatch_, L.numExt(), L.entries, L.numActive, L.scratch, L.scratchBytes, stream_);
   if (s != PVGPU_OK && err.empty()) err = fmt("layer \"", L.name, "\": ") + pvgpu_last_error();
   return s;
}

// HyPerCol::advanceTime: per phase, every layer of the phase receives its synaptic input (GSyn
// zeroed, then each incoming connection delivers into its channel), then updates and publishes.
pvgpu_status Column::step(std::string &err) {
   t_++;
   for (int phase = 0; phase <= maxPhase_; phase++) {
      std::vector<Layer *> now;
      for (auto &L : layers_)
         if (L->phase == phase) now.push_back(L.get());
      for (Layer *L : now) {
         if (L->kind == Layer::Input) continue;
         const size_t chan = (size_t)L->numRes() * nbatch_;
         if (cudaMemsetAsync(L->gsyn, 0, chan * L->numChannels * 4, stream_) != cudaSuccess) return PVGPU_ERR_LAUNCH;
         for (Conn *c : L->incoming) {
            if ((!c->W && !c->postPerspective) || (c->postPerspective && !c->Wpost)) {
               if (c->keyword != "IdentConn") {
                  err = fmt("connection \"", c->name, "\" has no weights (set_weights on it or its original)");
                  return PVGPU_ERR_BAD_ARG;
               }
            }
            pvgpu_status s = c->delivery->deliver(L->gsyn + chan * c->channel, stream_);
            if (s != PVGPU_OK) {
               err = fmt("connection \"", c->name, "\": ") + c->delivery->keyword() + ": " + pvgpu_last_error();
               return s;
            }
         }
      }
      for (Layer *L : now) {
         pvgpu_status s = update(*L, err);
         if (s != PVGPU_OK) return s;
      }
      for (Layer *L : now) {
         pvgpu_status s = output(*L, t_ * dt_, err);
         if (s != PVGPU_OK) return s;
      }
   }
   return PVGPU_OK;
}

pvgpu_status Column::advance(int numSteps, std::string &err) {
   if (numSteps < 0) return PVGPU_ERR_BAD_ARG;
   if (t_ == 0 && !initialOutputDone_ && !outputPath_.empty()) {
      // the initial conditions (HyPerCol::allocateDataStructures, columns/HyPerCol.cpp:400-415)
      initialOutputDone_ = true;
      for (auto &L : layers_) {
         if (L->kind == Layer::Input && !L->frames) continue;
         if (L->kind == Layer::Input) {
            pvgpu_status s = update(*L, err);  // the frame shown at time 0
            if (s != PVGPU_OK) return s;
         }
         pvgpu_status s = output(*L, 0.0, err);
         if (s != PVGPU_OK) return s;
      }
   }
   for (int i = 0; i < numSteps; i++) {
      pvgpu_status s = step(err);
      if (s != PVGPU_OK) return s;
   }
   if (cudaStreamSynchronize(stream_) != cudaSuccess) {
      err = "a kernel failed on the device";
      return PVGPU_ERR_LAUNCH;
   }
   return PVGPU_OK;
}

pvgpu_status Column::read(const std::string &name, int which, float *host, int64_t n, std::string &err) {
   Layer *L = layer(name);
   if (!L || !host || (which != 0 && which != 1) || (which == 0 && L->kind == Layer::Input)) {
      err = fmt("read: \"", name, "\" (which = 0 for V, 1 for A)");
      return PVGPU_ERR_BAD_ARG;
   }
   const int64_t nr = L->numRes() * nbatch_;
   if (n != nr) {
      err = "read: the host buffer must hold nbatch * ny * nx * nf floats";
      return PVGPU_ERR_BAD_ARG;
   }
   if (which == 0) {
      if (cudaMemcpy(host, L->V, nr * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return PVGPU_ERR_LAUNCH;
      return PVGPU_OK;
   }
   // restricted part of the extended activity
   const pvgpu_loc &l = L->loc;
   const int nxE = l.nx + l.halo.lt + l.halo.rt;
   const int nyE = l.ny + l.halo.dn + l.halo.up;
   std::vector<float> ext((size_t)L->numExt() * nbatch_);
   if (cudaMemcpy(ext.data(), L->A, ext.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return PVGPU_ERR_LAUNCH;
   for (int b = 0; b < nbatch_; b++)
      for (int y = 0; y < l.ny; y++)
         std::memcpy(host + (((size_t)b * l.ny + y) * l.nx) * l.nf,
                     ext.data() + (((size_t)b * nyE + y + l.halo.up) * nxE + l.halo.lt) * l.nf, (size_t)l.nx * l.nf * 4);
   return PVGPU_OK;
}

}  // namespace pvhost
