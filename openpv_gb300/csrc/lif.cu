// lif.cu -- LIF membrane update on the device (components/LIFActivityComponent.cpp:332-942, which
// the reference runs on the CPU only) and the Tausworthe generator of its noise
// (utils/cl_random.c).
//
// One thread per restricted neuron: noise on the EXC / INH / INHB GSyn channels, conductance and
// membrane update by the layer's method ('a' arma filter, 'b' Heun, 'o' exponential Euler), the
// threshold relaxation and the spike.  Every multiply, add and divide is a separately rounded
// float operation in the reference's order (no contraction), the generator is integer-exact, and
// the per-launch decay factors exp(-dt/tau*) are computed on the host with the C library's expf
// as the reference does; so 'b', whose per-neuron arithmetic has no transcendental, equals the
// reference bit for bit, and 'a' / 'o' differ only by the device's expf / powf / logf (within a
// few ulp) in their per-neuron filter coefficients.  Memory-bound: 88 bytes per neuron per step.
#include "pvgpu_internal.cuh"

#include <cmath>

namespace {

struct LifConst {
   pvgpu_lif_params p;
   float dt, dtSec, eE, eI, eIB, eVth;
   int numNeurons, total, nx, ny, nf, lt, rt, dn, up, numExt;
};

__device__ __forceinline__ uint32_t taus_component(uint32_t s, int a, int b, uint32_t mask, int d) {
   return ((s & mask) << d) ^ (((s << a) ^ s) >> b);
}

__device__ __forceinline__ uint4 taus_next(uint4 t) {
   t.y = taus_component(t.y, 13, 19, 4294967294u, 12);
   t.z = taus_component(t.z, 2, 25, 4294967288u, 4);
   t.w = taus_component(t.w, 3, 11, 4294967280u, 17);
   t.x = t.y ^ t.z ^ t.w;
   return t;
}

// the last output scaled to [0, 1): a float conversion, then an exact scaling by 2^-32
__device__ __forceinline__ float taus_uniform(uint4 t) { return __fmul_rn(__uint2float_rn(t.x), 2.3283064365386963e-10f); }

__device__ __forceinline__ float noise(uint4 &r, float gsyn, float dtSec, float freq, float amp) {
   r = taus_next(r);
   if (taus_uniform(r) < __fmul_rn(dtSec, freq)) {
      r = taus_next(r);
      gsyn = __fadd_rn(gsyn, __fmul_rn(amp, taus_uniform(r)));
   }
   return gsyn;
}

__device__ __forceinline__ float add4(float a, float b, float c, float d) {
   return __fadd_rn(__fadd_rn(__fadd_rn(a, b), c), d);
}

// (Vrest + Vexc*ge + Vinh*gi + VinhB*gib) / (1 + ge + gi + gib), left to right
__device__ __forceinline__ float v_inf(const pvgpu_lif_params &p, float ge, float gi, float gib) {
   float num = __fadd_rn(__fadd_rn(__fadd_rn(p.Vrest, __fmul_rn(p.Vexc, ge)), __fmul_rn(p.Vinh, gi)),
                         __fmul_rn(p.VinhB, gib));
   return __fdiv_rn(num, add4(1.0f, ge, gi, gib));
}

__device__ __forceinline__ float dvdt(const pvgpu_lif_params &p, float v, float ge, float gi, float gib) {
   float g = add4(1.0f, ge, gi, gib);
   float num = __fadd_rn(__fadd_rn(__fadd_rn(p.Vrest, __fmul_rn(p.Vexc, ge)), __fmul_rn(p.Vinh, gi)),
                         __fmul_rn(p.VinhB, gib));
   float vinf = __fdiv_rn(num, g);
   return __fdiv_rn(__fmul_rn(g, __fadd_rn(vinf, -v)), p.tau);
}

template <char M>
__global__ void __launch_bounds__(256) lif_kernel(LifConst c, uint4 *__restrict__ rnd, float *__restrict__ V,
                                                  float *__restrict__ Vth, float *__restrict__ GE,
                                                  float *__restrict__ GI, float *__restrict__ GIB,
                                                  const float *__restrict__ gsyn, float *__restrict__ aExt) {
   const float GMAX = 10.0f;
   const pvgpu_lif_params &p = c.p;
   for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < c.total; k += gridDim.x * blockDim.x) {
      const int b = k / c.numNeurons, kr = k - b * c.numNeurons;
      const int f = kr % c.nf, x = (kr / c.nf) % c.nx, y = kr / (c.nf * c.nx);
      const int64_t kex = (int64_t)b * c.numExt + ((int64_t)(y + c.up) * (c.nx + c.lt + c.rt) + (x + c.lt)) * c.nf + f;
      uint4 r = rnd[k];
      float v = V[k], vth = Vth[k], ge = GE[k], gi = GI[k], gib = GIB[k];
      const float inE = noise(r, gsyn[k], c.dtSec, p.noiseFreqE, p.noiseAmpE);
      const float inI = noise(r, gsyn[c.total + k], c.dtSec, p.noiseFreqI, p.noiseAmpI);
      const float inIB = noise(r, gsyn[2 * (int64_t)c.total + k], c.dtSec, p.noiseFreqIB, p.noiseAmpIB);
      if (M == 'o') {
         ge = fminf(__fadd_rn(inE, __fmul_rn(ge, c.eE)), GMAX);
         gi = fminf(__fadd_rn(inI, __fmul_rn(gi, c.eI)), GMAX);
         gib = fminf(__fadd_rn(inIB, __fmul_rn(gib, c.eIB)), GMAX);
         const float tauInf = __fmul_rn(__fdiv_rn(c.dt, p.tau), add4(1.0f, ge, gi, gib));
         const float vInf = v_inf(p, ge, gi, gib);
         v = __fadd_rn(vInf, __fmul_rn(__fadd_rn(v, -vInf), expf(-tauInf)));
      } else {
         float ge0 = __fadd_rn(ge, inE), gi0 = __fadd_rn(gi, inI), gib0 = __fadd_rn(gib, inIB);
         float tauInf0 = 0.0f, vInf0 = 0.0f;
         if (M == 'a') {  // before the cap
            tauInf0 = __fdiv_rn(p.tau, add4(1.0f, ge0, gi0, gib0));
            vInf0 = v_inf(p, ge0, gi0, gib0);
         }
         ge0 = fminf(ge0, GMAX);
         gi0 = fminf(gi0, GMAX);
         gib0 = fminf(gib0, GMAX);
         const float ge1 = __fmul_rn(ge0, c.eE), gi1 = __fmul_rn(gi0, c.eI), gib1 = __fmul_rn(gib0, c.eIB);
         if (M == 'b') {
            const float d1 = dvdt(p, v, ge0, gi0, gib0);
            const float d2 = dvdt(p, __fadd_rn(v, __fmul_rn(c.dt, d1)), ge1, gi1, gib1);
            v = __fadd_rn(v, __fmul_rn(c.dt, __fmul_rn(__fadd_rn(d1, d2), 0.5f)));
         } else {
            // the end-of-step time constant takes the start-of-step G_IB, as the reference does
            const float tauInf1 = __fdiv_rn(p.tau, add4(1.0f, ge1, gi1, gib0));
            const float vInf1 = v_inf(p, ge1, gi1, gib1);
            const float slope = __fdiv_rn(__fadd_rn(tauInf1, -tauInf0), c.dt);
            const float ratio = __fdiv_rn(tauInf1, tauInf0);
            const float f1 = slope == 0.0f ? expf(-__fdiv_rn(c.dt, tauInf0)) : powf(ratio, __fdiv_rn(-1.0f, slope));
            const float f2 = slope == -1.0f
                                   ? __fmul_rn(__fdiv_rn(tauInf0, c.dt), logf(__fadd_rn(ratio, 1.0f)))
                                   : __fdiv_rn(__fadd_rn(1.0f, -__fmul_rn(__fdiv_rn(tauInf0, c.dt), __fadd_rn(1.0f, -f1))),
                                               __fadd_rn(1.0f, slope));
            const float f3 = __fadd_rn(__fadd_rn(1.0f, -f1), -f2);
            v = __fadd_rn(__fadd_rn(__fmul_rn(f1, v), __fmul_rn(f2, vInf0)), __fmul_rn(f3, vInf1));
         }
         ge = ge1;
         gi = gi1;
         gib = gib1;
      }
      vth = __fadd_rn(p.VthRest, __fmul_rn(__fadd_rn(vth, -p.VthRest), c.eVth));
      const bool fired = v > vth;
      aExt[kex] = fired ? 1.0f : 0.0f;
      if (fired) {
         v = p.Vrest;
         vth = __fadd_rn(vth, p.deltaVth);
         gib = __fadd_rn(gib, p.deltaGIB);
      }
      rnd[k] = r;
      V[k] = v;
      Vth[k] = vth;
      GE[k] = ge;
      GI[k] = gi;
      GIB[k] = gib;
   }
}

// cl_random_init: element i seeded with i + seed (0 counts as 1), three LCG steps, six warm-up
// generator steps, s0 = s1 ^ s2 ^ s3
__global__ void taus_init_kernel(uint4 *state, int64_t count, uint32_t seed) {
   for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
      uint32_t s = (uint32_t)i + seed;
      if (s == 0) s = 1;
      uint4 t;
      t.y = 69069u * s;
      t.z = 69069u * t.y;
      t.w = 69069u * t.z;
      for (int w = 0; w < 6; w++) t = taus_next(t);
      t.x = t.y ^ t.z ^ t.w;
      state[i] = t;
   }
}

int grid_for(int64_t n) {
   int dev = 0, sms = 148;
   cudaGetDevice(&dev);
   cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   const int64_t blocks = (n + 255) / 256;
   return (int)(blocks < (int64_t)sms * 8 ? (blocks > 0 ? blocks : 1) : (int64_t)sms * 8);
}

}  // namespace

extern "C" pvgpu_status pvgpu_lif_update(const pvgpu_loc *loc, char method, const pvgpu_lif_params *params, float dt,
                                         pvgpu_taus *rnd, float *V, float *Vth, float *GE, float *GI, float *GIB,
                                         const float *gsynHead, float *aExt, void *stream) {
   if (!loc || !params || !rnd || !V || !Vth || !GE || !GI || !GIB || !gsynHead || !aExt || !pvgpu::loc_valid(*loc))
      return PVGPU_ERR_BAD_ARG;
   if (method != 'a' && method != 'b' && method != 'o') return PVGPU_ERR_BAD_ARG;
   LifConst c;
   c.p = *params;
   c.dt = dt;
   c.dtSec = 0.001f * dt;
   // host expf, as the reference computes these once per update
   c.eE = std::exp(-dt / params->tauE);
   c.eI = std::exp(-dt / params->tauI);
   c.eIB = std::exp(-dt / params->tauIB);
   c.eVth = std::exp(-dt / params->tauVth);
   c.nx = loc->nx;
   c.ny = loc->ny;
   c.nf = loc->nf;
   c.lt = loc->halo.lt;
   c.rt = loc->halo.rt;
   c.dn = loc->halo.dn;
   c.up = loc->halo.up;
   const int64_t numNeurons = (int64_t)loc->nx * loc->ny * loc->nf;
   const int64_t total = numNeurons * loc->nbatch;
   const int64_t numExt = (int64_t)(loc->nx + c.lt + c.rt) * (loc->ny + c.dn + c.up) * loc->nf;
   if (total > 0x7fffffff || numExt > 0x7fffffff) return PVGPU_ERR_UNSUPPORTED_SHAPE;
   c.numNeurons = (int)numNeurons;
   c.total = (int)total;
   c.numExt = (int)numExt;
   cudaStream_t s = pvgpu::as_stream(stream);
   uint4 *r = reinterpret_cast<uint4 *>(rnd);
   const int grid = grid_for(total);
   if (method == 'a') lif_kernel<'a'><<<grid, 256, 0, s>>>(c, r, V, Vth, GE, GI, GIB, gsynHead, aExt);
   else if (method == 'b') lif_kernel<'b'><<<grid, 256, 0, s>>>(c, r, V, Vth, GE, GI, GIB, gsynHead, aExt);
   else lif_kernel<'o'><<<grid, 256, 0, s>>>(c, r, V, Vth, GE, GI, GIB, gsynHead, aExt);
   PVGPU_CHECK_LAUNCH("lif_update");
   return PVGPU_OK;
}

extern "C" pvgpu_status pvgpu_taus_init(pvgpu_taus *state, int64_t count, uint32_t seed, void *stream) {
   if (!state || count < 0) return PVGPU_ERR_BAD_ARG;
   if (count == 0) return PVGPU_OK;
   taus_init_kernel<<<grid_for(count), 256, 0, pvgpu::as_stream(stream)>>>(reinterpret_cast<uint4 *>(state), count,
                                                                         seed == 0 ? 1u : seed);
   PVGPU_CHECK_LAUNCH("taus_init");
   return PVGPU_OK;
}
