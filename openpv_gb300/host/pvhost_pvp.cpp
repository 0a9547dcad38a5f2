// pvhost_pvp.cpp -- the .pvp part of the C API of include/pvhost.h: pvhost::PvpWriter / PvpReader
// with frame payloads packed and unpacked on the device (pvgpu_pvp_*), so that only the entries
// a sparse file holds cross PCIe / C2C.
#include "pvhost.h"

#include "pvp.hpp"

#include <cuda_runtime.h>

#include <new>
#include <string>
#include <vector>

// error text shared with the rest of the C API (pvhost_capi.cpp)
namespace pvhost_capi {
pvgpu_status fail(pvgpu_status s, const std::string &msg);
}
using pvhost_capi::fail;

struct pvhost_pvp_writer {
   pvhost::PvpWriter w;
   void *dev = nullptr;  // packed frames: entries (sparse) or restricted values (dense)
   size_t devBytes = 0;
   int32_t *devCounts = nullptr;
   std::vector<unsigned char> host;
   ~pvhost_pvp_writer() {
      if (dev) cudaFree(dev);
      if (devCounts) cudaFree(devCounts);
   }
};

struct pvhost_pvp_reader {
   pvhost::PvpReader r;
};

namespace {

pvgpu_status cuda_fail(cudaError_t e, const char *where) {
   return fail(PVGPU_ERR_LAUNCH, std::string(where) + ": " + cudaGetErrorString(e));
}

bool same_size(const pvhost::PvpHeader &h, const pvgpu_loc &l) { return h.nx == l.nx && h.ny == l.ny && h.nf == l.nf; }

}  // namespace

extern "C" pvgpu_status pvhost_pvp_writer_open(const char *path, int nx, int ny, int nf, int sparse,
                                               pvhost_pvp_writer **out) {
   if (!path || !out) return fail(PVGPU_ERR_BAD_ARG, "null argument");
   auto *w = new (std::nothrow) pvhost_pvp_writer;
   if (!w) return fail(PVGPU_ERR_OOM, "out of host memory");
   std::string err;
   if (!w->w.open(path, nx, ny, nf, sparse != 0, err)) {
      delete w;
      return fail(PVGPU_ERR_BAD_ARG, err);
   }
   *out = w;
   return PVGPU_OK;
}

static pvgpu_status ensure_device(pvhost_pvp_writer *w, size_t bytes, int nbatch) {
   if (w->devBytes < bytes) {
      if (w->dev) cudaFree(w->dev);
      w->dev = nullptr;
      w->devBytes = 0;
      cudaError_t e = cudaMalloc(&w->dev, bytes);
      if (e != cudaSuccess) return cuda_fail(e, "pvp writer buffer");
      w->devBytes = bytes;
      if (w->devCounts) cudaFree(w->devCounts);
      w->devCounts = nullptr;
   }
   if (!w->devCounts) {
      cudaError_t e = cudaMalloc(&w->devCounts, sizeof(int32_t) * (size_t)(nbatch > 0 ? nbatch : 1) * 64);
      if (e != cudaSuccess) return cuda_fail(e, "pvp writer counts");
   }
   return PVGPU_OK;
}

extern "C" pvgpu_status pvhost_pvp_write_sparse_device(pvhost_pvp_writer *w, const pvgpu_loc *loc,
                                                       const pvgpu_entry *entries, const int64_t *numActive,
                                                       double timestamp, void *stream) {
   if (!w || !loc || !entries || !numActive) return fail(PVGPU_ERR_BAD_ARG, "null argument");
   if (!w->w.sparse() || !same_size(w->w.header(), *loc)) return fail(PVGPU_ERR_BAD_ARG, "file and layer differ");
   if (loc->nbatch > 64) return fail(PVGPU_ERR_UNSUPPORTED_SHAPE, "more than 64 batch elements per call");
   const size_t nRes = (size_t)loc->nx * loc->ny * loc->nf;
   pvgpu_status st = ensure_device(w, nRes * sizeof(pvgpu_entry) * (size_t)loc->nbatch, loc->nbatch);
   if (st != PVGPU_OK) return st;
   auto *packed = static_cast<pvgpu_entry *>(w->dev);
   st = pvgpu_pvp_sparse_frames(loc, entries, numActive, packed, w->devCounts, stream);
   if (st != PVGPU_OK) return fail(st, std::string("pvgpu_pvp_sparse_frames: ") + pvgpu_last_error());
   cudaStream_t s = static_cast<cudaStream_t>(stream);
   std::vector<int32_t> counts((size_t)loc->nbatch);
   cudaError_t e = cudaMemcpyAsync(counts.data(), w->devCounts, sizeof(int32_t) * counts.size(),
                                   cudaMemcpyDeviceToHost, s);
   if (e == cudaSuccess) e = cudaStreamSynchronize(s);
   if (e != cudaSuccess) return cuda_fail(e, "pvp counts copy");
   std::string err;
   for (int b = 0; b < loc->nbatch; b++) {
      const size_t c = (size_t)(counts[(size_t)b] > 0 ? counts[(size_t)b] : 0);
      w->host.resize(c * sizeof(pvgpu_entry) + 1);
      if (c > 0) {
         e = cudaMemcpyAsync(w->host.data(), packed + (size_t)b * nRes, c * sizeof(pvgpu_entry), cudaMemcpyDeviceToHost, s);
         if (e == cudaSuccess) e = cudaStreamSynchronize(s);
         if (e != cudaSuccess) return cuda_fail(e, "pvp entries copy");
      }
      if (!w->w.write_sparse(timestamp, reinterpret_cast<const pvgpu_entry *>(w->host.data()), (int32_t)c, err))
         return fail(PVGPU_ERR_BAD_ARG, err);
   }
   return PVGPU_OK;
}

extern "C" pvgpu_status pvhost_pvp_write_dense_device(pvhost_pvp_writer *w, const pvgpu_loc *loc, const float *aExt,
                                                      double timestamp, void *stream) {
   if (!w || !loc || !aExt) return fail(PVGPU_ERR_BAD_ARG, "null argument");
   if (w->w.sparse() || !same_size(w->w.header(), *loc)) return fail(PVGPU_ERR_BAD_ARG, "file and layer differ");
   const size_t nRes = (size_t)loc->nx * loc->ny * loc->nf;
   pvgpu_status st = ensure_device(w, nRes * sizeof(float) * (size_t)loc->nbatch, loc->nbatch);
   if (st != PVGPU_OK) return st;
   st = pvgpu_pvp_dense_frames(loc, aExt, static_cast<float *>(w->dev), stream);
   if (st != PVGPU_OK) return fail(st, std::string("pvgpu_pvp_dense_frames: ") + pvgpu_last_error());
   cudaStream_t s = static_cast<cudaStream_t>(stream);
   w->host.resize(nRes * sizeof(float) * (size_t)loc->nbatch);
   cudaError_t e = cudaMemcpyAsync(w->host.data(), w->dev, w->host.size(), cudaMemcpyDeviceToHost, s);
   if (e == cudaSuccess) e = cudaStreamSynchronize(s);
   if (e != cudaSuccess) return cuda_fail(e, "pvp frame copy");
   std::string err;
   for (int b = 0; b < loc->nbatch; b++)
      if (!w->w.write_dense(timestamp, reinterpret_cast<const float *>(w->host.data()) + (size_t)b * nRes, err))
         return fail(PVGPU_ERR_BAD_ARG, err);
   return PVGPU_OK;
}

extern "C" pvgpu_status pvhost_pvp_write_sparse_host(pvhost_pvp_writer *w, const pvgpu_entry *entries, int32_t count,
                                                     double timestamp) {
   if (!w) return fail(PVGPU_ERR_BAD_ARG, "null writer");
   std::string err;
   if (!w->w.write_sparse(timestamp, entries, count, err)) return fail(PVGPU_ERR_BAD_ARG, err);
   return PVGPU_OK;
}

extern "C" pvgpu_status pvhost_pvp_write_dense_host(pvhost_pvp_writer *w, const float *restricted, double timestamp) {
   if (!w || !restricted) return fail(PVGPU_ERR_BAD_ARG, "null argument");
   std::string err;
   if (!w->w.write_dense(timestamp, restricted, err)) return fail(PVGPU_ERR_BAD_ARG, err);
   return PVGPU_OK;
}

extern "C" pvgpu_status pvhost_pvp_writer_close(pvhost_pvp_writer *w) {
   if (!w) return PVGPU_OK;
   std::string err;
   const bool ok = w->w.close(err);
   delete w;
   return ok ? PVGPU_OK : fail(PVGPU_ERR_BAD_ARG, err);
}

extern "C" pvgpu_status pvhost_pvp_reader_open(const char *path, pvhost_pvp_reader **out) {
   if (!path || !out) return fail(PVGPU_ERR_BAD_ARG, "null argument");
   auto *r = new (std::nothrow) pvhost_pvp_reader;
   if (!r) return fail(PVGPU_ERR_OOM, "out of host memory");
   std::string err;
   if (!r->r.open(path, err)) {
      delete r;
      return fail(PVGPU_ERR_BAD_ARG, err);
   }
   *out = r;
   return PVGPU_OK;
}

extern "C" pvgpu_status pvhost_pvp_reader_info(pvhost_pvp_reader *r, int32_t *out18, double *timestamp,
                                               int *numFrames) {
   if (!r) return fail(PVGPU_ERR_BAD_ARG, "null reader");
   const pvhost::PvpHeader &h = r->r.header();
   if (out18) {
      const int32_t v[18] = {h.headerSize, h.numParams, h.fileType,   h.nx,         h.ny,  h.nf,
                             h.numRecords, h.recordSize, h.dataSize,  h.dataType,   h.nxProcs, h.nyProcs,
                             h.nxExtended, h.nyExtended, h.kx0,       h.ky0,        h.nBatch,  h.nBands};
      for (int i = 0; i < 18; i++) out18[i] = v[i];
   }
   if (timestamp) *timestamp = h.timestamp;
   if (numFrames) *numFrames = r->r.num_frames();
   return PVGPU_OK;
}

extern "C" pvgpu_status pvhost_pvp_read_dense(pvhost_pvp_reader *r, int frame, float *host, int64_t n,
                                              double *timestamp) {
   if (!r || !host) return fail(PVGPU_ERR_BAD_ARG, "null argument");
   const pvhost::PvpHeader &h = r->r.header();
   if (n != (int64_t)h.nx * h.ny * h.nf) return fail(PVGPU_ERR_BAD_ARG, "buffer size differs from nx*ny*nf");
   std::string err;
   if (!r->r.read_dense(frame, host, timestamp, err)) return fail(PVGPU_ERR_BAD_ARG, err);
   return PVGPU_OK;
}

extern "C" pvgpu_status pvhost_pvp_read_sparse(pvhost_pvp_reader *r, int frame, pvgpu_entry *host, int64_t capacity,
                                               int32_t *count, double *timestamp) {
   if (!r || !count) return fail(PVGPU_ERR_BAD_ARG, "null argument");
   std::vector<pvgpu_entry> e;
   std::string err;
   if (!r->r.read_sparse(frame, e, timestamp, err)) return fail(PVGPU_ERR_BAD_ARG, err);
   if ((int64_t)e.size() > capacity || (!host && !e.empty())) return fail(PVGPU_ERR_BAD_ARG, "buffer too small");
   for (size_t i = 0; i < e.size(); i++) host[i] = e[i];
   *count = (int32_t)e.size();
   return PVGPU_OK;
}

extern "C" pvgpu_status pvhost_pvp_read_to_device(pvhost_pvp_reader *r, int firstFrame, const pvgpu_loc *loc,
                                                  float *aExt, void *stream) {
   if (!r || !loc || !aExt) return fail(PVGPU_ERR_BAD_ARG, "null argument");
   const pvhost::PvpHeader &h = r->r.header();
   if (!same_size(h, *loc)) return fail(PVGPU_ERR_BAD_ARG, "file and layer differ");
   if (firstFrame < 0 || firstFrame + loc->nbatch > r->r.num_frames()) return fail(PVGPU_ERR_BAD_ARG, "frame range");
   const size_t nRes = (size_t)loc->nx * loc->ny * loc->nf;
   // every batch element as entries, one upload, one scatter on the device
   std::vector<pvgpu_entry> all(nRes * (size_t)loc->nbatch);
   std::vector<int32_t> counts((size_t)loc->nbatch);
   std::string err;
   for (int b = 0; b < loc->nbatch; b++) {
      std::vector<pvgpu_entry> e;
      if (!r->r.read_sparse(firstFrame + b, e, nullptr, err)) return fail(PVGPU_ERR_BAD_ARG, err);
      counts[(size_t)b] = (int32_t)e.size();
      for (size_t i = 0; i < e.size(); i++) all[(size_t)b * nRes + i] = e[i];
   }
   cudaStream_t s = static_cast<cudaStream_t>(stream);
   pvgpu_entry *dE = nullptr;
   int32_t *dC = nullptr;
   cudaError_t ce = cudaMalloc(&dE, sizeof(pvgpu_entry) * all.size());
   if (ce == cudaSuccess) ce = cudaMalloc(&dC, sizeof(int32_t) * (counts.size() + 1));
   if (ce == cudaSuccess)
      ce = cudaMemcpyAsync(dE, all.data(), sizeof(pvgpu_entry) * all.size(), cudaMemcpyHostToDevice, s);
   if (ce == cudaSuccess)
      ce = cudaMemcpyAsync(dC, counts.data(), sizeof(int32_t) * counts.size(), cudaMemcpyHostToDevice, s);
   if (ce == cudaSuccess) ce = cudaMemsetAsync(dC + counts.size(), 0, sizeof(int32_t), s);
   pvgpu_status st = PVGPU_OK;
   if (ce == cudaSuccess) st = pvgpu_pvp_scatter_sparse(loc, dE, dC, aExt, dC + counts.size(), stream);
   int32_t bad = 0;
   if (ce == cudaSuccess && st == PVGPU_OK)
      ce = cudaMemcpyAsync(&bad, dC + counts.size(), sizeof(int32_t), cudaMemcpyDeviceToHost, s);
   if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
   if (dE) cudaFree(dE);
   if (dC) cudaFree(dC);
   if (ce != cudaSuccess) return cuda_fail(ce, "pvp read to device");
   if (st != PVGPU_OK) return fail(st, std::string("pvgpu_pvp_scatter_sparse: ") + pvgpu_last_error());
   if (bad) return fail(PVGPU_ERR_BAD_ARG, "pvp frame entry outside the layer");
   return PVGPU_OK;
}

extern "C" pvgpu_status pvhost_pvp_reader_close(pvhost_pvp_reader *r) {
   delete r;
   return PVGPU_OK;
}
