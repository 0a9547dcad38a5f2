// ref_lif_shim.cpp -- C entry points that run the reference's own LIF update loops
// (LIFActivityComponent::updateActivityArma / Beginning / Original, compiled unmodified from the
// reference tree against the stand-in oracle/refshim/LIFActivityComponent.hpp) and its
// Tausworthe generator (utils/cl_random.c, compiled unmodified).  TEST INFRASTRUCTURE ONLY
// (oracle/_ref).
#include "LIFActivityComponent.hpp"

#include <cstring>

namespace {
// The update loops are protected members that use only their arguments.
struct LIFAccess : PV::LIFActivityComponent {
   using PV::LIFActivityComponent::updateActivityArma;
   using PV::LIFActivityComponent::updateActivityBeginning;
   using PV::LIFActivityComponent::updateActivityOriginal;
   LIFAccess() {}
};
static_assert(sizeof(PV::LIFParams) == 18 * sizeof(float), "LIFParams is 18 floats");
static_assert(sizeof(taus_uint4) == 4 * sizeof(unsigned int), "taus_uint4 is 4 words");
}  // namespace

extern "C" {

struct pvr_loc3 {
   int nbatch, nx, ny, nf;
   int lt, rt, dn, up;
};

// params18: LIFParams in declaration order (Vrest, Vexc, Vinh, VinhB, VthRest, tau, tauVth,
// deltaVth, deltaGIB, noiseAmpE, noiseAmpI, noiseAmpIB, noiseFreqE, noiseFreqI, noiseFreqIB,
// tauE, tauI, tauIB).  gsynHead: the EXC, INH, INHB channels, each nbatch * nx*ny*nf.
int pvr_lif_update(char method, pvr_loc3 const *l, float const *params18, float simTime, float dt, void *rnd,
                   float *V, float *Vth, float *GE, float *GI, float *GIB, float const *gsynHead, float *A) {
   PV::LIFParams p;
   std::memcpy(&p, params18, sizeof(p));
   LIFAccess lif;
   int n = l->nx * l->ny * l->nf;
   taus_uint4 *r = static_cast<taus_uint4 *>(rnd);
   switch (method) {
      case 'a':
         lif.updateActivityArma(l->nbatch, n, simTime, dt, l->nx, l->ny, l->nf, l->lt, l->rt, l->dn, l->up, &p, r, V,
                                Vth, GE, GI, GIB, gsynHead, A);
         return 0;
      case 'b':
         lif.updateActivityBeginning(l->nbatch, n, simTime, dt, l->nx, l->ny, l->nf, l->lt, l->rt, l->dn, l->up, &p,
                                     r, V, Vth, GE, GI, GIB, gsynHead, A);
         return 0;
      case 'o':
         lif.updateActivityOriginal(l->nbatch, n, simTime, dt, l->nx, l->ny, l->nf, l->lt, l->rt, l->dn, l->up, &p,
                                    r, V, Vth, GE, GI, GIB, gsynHead, A);
         return 0;
      default: return -1;
   }
}

void pvr_taus_init(void *state, size_t count, unsigned int seed) {
   cl_random_init(static_cast<taus_uint4 *>(state), count, seed);
}

void pvr_taus_next(void *state, size_t count) {
   taus_uint4 *s = static_cast<taus_uint4 *>(state);
   for (size_t i = 0; i < count; i++) s[i] = cl_random_get(s[i]);
}

}  // extern "C"
