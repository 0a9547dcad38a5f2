// pvp.hpp -- OpenPV .pvp activity files on the host: the 80-byte activity header
// (utils/BufferUtilsPvp.hpp:73-77), dense frames (PVP_NONSPIKING_ACT_FILE_TYPE = 4: a double
// timestamp, then nx*ny*nf floats, io/LayerIO.cpp:81-95), sparse-values frames
// (PVP_ACT_SPARSEVALUES_FILE_TYPE = 6: a double timestamp, an int count, then count
// {uint32 restricted index, float value} entries, io/SparseLayerIO.cpp:95-119) and, for reading
// only, binary spike frames (PVP_ACT_FILE_TYPE = 2: timestamp, count, count uint32 indices, every
// value 1).  The writer follows LayerIO / SparseLayerIO::writeHeader: header once with
// nBands = 0 and timestamp 0, frames appended, and nBands (byte 68) rewritten after every frame.
#pragma once

#include "pvgpu.h"

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace pvhost {

struct PvpHeader {
   int32_t headerSize, numParams, fileType, nx, ny, nf, numRecords, recordSize, dataSize, dataType, nxProcs, nyProcs,
         nxExtended, nyExtended, kx0, ky0, nBatch, nBands;
   double timestamp;
};
static_assert(sizeof(PvpHeader) == 80, "pvp activity header is 80 bytes");

constexpr int kPvpBinary = 2, kPvpDense = 4, kPvpSparseValues = 6;

class PvpWriter {
 public:
   ~PvpWriter();
   bool open(const std::string &path, int nx, int ny, int nf, bool sparse, std::string &err);
   bool write_dense(double timestamp, const float *restrictedValues, std::string &err);
   bool write_sparse(double timestamp, const pvgpu_entry *entries, int32_t count, std::string &err);
   bool close(std::string &err);
   bool sparse() const { return h_.fileType == kPvpSparseValues; }
   const PvpHeader &header() const { return h_; }

 private:
   bool finish_frame(std::string &err);
   FILE *f_ = nullptr;
   PvpHeader h_{};
   std::string path_;
};

class PvpReader {
 public:
   ~PvpReader();
   bool open(const std::string &path, std::string &err);
   const PvpHeader &header() const { return h_; }
   int num_frames() const { return (int)starts_.size(); }
   // A frame as the restricted activity [ny][nx][nf] (sparse and binary frames expanded).
   bool read_dense(int frame, float *out, double *timestamp, std::string &err);
   // A frame as {restricted index, value} entries in file order (dense frames: nonzeros in index
   // order; binary frames: value 1).
   bool read_sparse(int frame, std::vector<pvgpu_entry> &out, double *timestamp, std::string &err);

 private:
   FILE *f_ = nullptr;
   PvpHeader h_{};
   std::vector<long> starts_;  // byte offset of each frame
   std::vector<int32_t> counts_;
};

}  // namespace pvhost
