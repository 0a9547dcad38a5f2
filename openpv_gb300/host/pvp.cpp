// pvp.cpp -- .pvp activity file reader and writer (see pvp.hpp).
#include "pvp.hpp"

#include <cstring>
#include <sstream>

namespace pvhost {

namespace {

std::string msg(const std::string &path, const char *what) {
   std::ostringstream o;
   o << "pvp \"" << path << "\": " << what;
   return o.str();
}

}  // namespace

// ---- writer ------------------------------------------------------------------------------

PvpWriter::~PvpWriter() {
   if (f_) std::fclose(f_);
}

bool PvpWriter::open(const std::string &path, int nx, int ny, int nf, bool sparse, std::string &err) {
   if (nx <= 0 || ny <= 0 || nf <= 0) {
      err = msg(path, "nonpositive layer size");
      return false;
   }
   path_ = path;
   f_ = std::fopen(path.c_str(), "wb");
   if (!f_) {
      err = msg(path, "cannot open for writing");
      return false;
   }
   // SparseLayerIO::writeHeader (io/SparseLayerIO.cpp:213-242) / LayerIO::writeHeader
   h_.headerSize = (int32_t)sizeof(PvpHeader);
   h_.numParams = 20;
   h_.fileType = sparse ? kPvpSparseValues : kPvpDense;
   h_.nx = nx;
   h_.ny = ny;
   h_.nf = nf;
   h_.numRecords = 1;
   h_.recordSize = sparse ? 0 : nx * ny * nf;
   h_.dataSize = sparse ? 8 : 4;
   h_.dataType = 3;  // BufferUtils::FLOAT
   h_.nxProcs = 1;
   h_.nyProcs = 1;
   h_.nxExtended = nx;
   h_.nyExtended = ny;
   h_.kx0 = 0;
   h_.ky0 = 0;
   h_.nBatch = 1;
   h_.nBands = 0;
   h_.timestamp = 0.0;
   if (std::fwrite(&h_, sizeof(h_), 1, f_) != 1) {
      err = msg(path, "header write failed");
      return false;
   }
   return true;
}

bool PvpWriter::finish_frame(std::string &err) {
   // nBands = frames written, at byte 68 (io/SparseLayerIO.cpp:200-211)
   h_.nBands++;
   if (std::fseek(f_, 68L, SEEK_SET) != 0 || std::fwrite(&h_.nBands, sizeof(int32_t), 1, f_) != 1 ||
       std::fseek(f_, 0L, SEEK_END) != 0) {
      err = msg(path_, "header update failed");
      return false;
   }
   return true;
}

bool PvpWriter::write_dense(double timestamp, const float *values, std::string &err) {
   if (!f_ || sparse()) {
      err = msg(path_, "not open as a dense file");
      return false;
   }
   const size_t n = (size_t)h_.nx * h_.ny * h_.nf;
   if (std::fwrite(&timestamp, sizeof(double), 1, f_) != 1 || std::fwrite(values, sizeof(float), n, f_) != n) {
      err = msg(path_, "frame write failed");
      return false;
   }
   return finish_frame(err);
}

bool PvpWriter::write_sparse(double timestamp, const pvgpu_entry *entries, int32_t count, std::string &err) {
   if (!f_ || !sparse()) {
      err = msg(path_, "not open as a sparse file");
      return false;
   }
   if (count < 0 || (count > 0 && !entries)) {
      err = msg(path_, "bad entry count");
      return false;
   }
   if (std::fwrite(&timestamp, sizeof(double), 1, f_) != 1 || std::fwrite(&count, sizeof(int32_t), 1, f_) != 1 ||
       (count > 0 && std::fwrite(entries, sizeof(pvgpu_entry), (size_t)count, f_) != (size_t)count)) {
      err = msg(path_, "frame write failed");
      return false;
   }
   return finish_frame(err);
}

bool PvpWriter::close(std::string &err) {
   if (!f_) return true;
   const bool ok = std::fclose(f_) == 0;
   f_ = nullptr;
   if (!ok) err = msg(path_, "close failed");
   return ok;
}

// ---- reader ------------------------------------------------------------------------------

PvpReader::~PvpReader() {
   if (f_) std::fclose(f_);
}

bool PvpReader::open(const std::string &path, std::string &err) {
   f_ = std::fopen(path.c_str(), "rb");
   if (!f_) {
      err = msg(path, "cannot open");
      return false;
   }
   if (std::fread(&h_, sizeof(h_), 1, f_) != 1) {
      err = msg(path, "short header");
      return false;
   }
   if (h_.headerSize < (int32_t)sizeof(PvpHeader) || h_.nx <= 0 || h_.ny <= 0 || h_.nf <= 0) {
      err = msg(path, "not an activity file");
      return false;
   }
   std::fseek(f_, 0L, SEEK_END);
   const long length = std::ftell(f_);
   const long n = (long)h_.nx * h_.ny * h_.nf;
   if (h_.fileType == kPvpDense) {
      if (h_.dataSize != 4) {
         err = msg(path, "dense frames must hold 4-byte floats");
         return false;
      }
      const long frameBytes = 8 + n * 4;
      for (long pos = h_.headerSize; pos + frameBytes <= length; pos += frameBytes) {
         starts_.push_back(pos);
         counts_.push_back((int32_t)n);
      }
   } else if (h_.fileType == kPvpSparseValues || h_.fileType == kPvpBinary) {
      const long entryBytes = h_.fileType == kPvpSparseValues ? 8 : 4;
      long pos = h_.headerSize;
      while (pos + 12 <= length) {
         int32_t count = -1;
         std::fseek(f_, pos + 8, SEEK_SET);
         if (std::fread(&count, sizeof(count), 1, f_) != 1 || count < 0 || count > n ||
             pos + 12 + count * entryBytes > length) {
            err = msg(path, "truncated or corrupt sparse frame");
            return false;
         }
         starts_.push_back(pos);
         counts_.push_back(count);
         pos += 12 + count * entryBytes;
      }
   } else {
      err = msg(path, "unsupported file type (activity files are types 2, 4 and 6)");
      return false;
   }
   return true;
}

bool PvpReader::read_sparse(int frame, std::vector<pvgpu_entry> &out, double *timestamp, std::string &err) {
   if (frame < 0 || frame >= num_frames()) {
      err = "pvp: frame index out of range";
      return false;
   }
   const long n = (long)h_.nx * h_.ny * h_.nf;
   std::fseek(f_, starts_[frame], SEEK_SET);
   double t = 0.0;
   if (std::fread(&t, sizeof(double), 1, f_) != 1) {
      err = "pvp: short frame";
      return false;
   }
   if (timestamp) *timestamp = t;
   out.clear();
   if (h_.fileType == kPvpDense) {
      std::vector<float> v((size_t)n);
      if (std::fread(v.data(), sizeof(float), (size_t)n, f_) != (size_t)n) {
         err = "pvp: short frame";
         return false;
      }
      for (long k = 0; k < n; k++)
         if (v[(size_t)k] != 0.0f) out.push_back(pvgpu_entry{(uint32_t)k, v[(size_t)k]});
      return true;
   }
   std::fseek(f_, 4, SEEK_CUR);  // count, known from the scan
   const int32_t count = counts_[frame];
   if (h_.fileType == kPvpSparseValues) {
      out.resize((size_t)count);
      if (count > 0 && std::fread(out.data(), sizeof(pvgpu_entry), (size_t)count, f_) != (size_t)count) {
         err = "pvp: short frame";
         return false;
      }
   } else {
      std::vector<uint32_t> idx((size_t)count);
      if (count > 0 && std::fread(idx.data(), sizeof(uint32_t), (size_t)count, f_) != (size_t)count) {
         err = "pvp: short frame";
         return false;
      }
      out.reserve((size_t)count);
      for (uint32_t k : idx) out.push_back(pvgpu_entry{k, 1.0f});
   }
   for (const pvgpu_entry &e : out)
      if ((long)e.index >= n) {
         err = "pvp: entry index outside the layer";
         return false;
      }
   return true;
}

bool PvpReader::read_dense(int frame, float *out, double *timestamp, std::string &err) {
   const long n = (long)h_.nx * h_.ny * h_.nf;
   if (h_.fileType == kPvpDense) {
      if (frame < 0 || frame >= num_frames()) {
         err = "pvp: frame index out of range";
         return false;
      }
      std::fseek(f_, starts_[frame], SEEK_SET);
      double t = 0.0;
      if (std::fread(&t, sizeof(double), 1, f_) != 1 || std::fread(out, sizeof(float), (size_t)n, f_) != (size_t)n) {
         err = "pvp: short frame";
         return false;
      }
      if (timestamp) *timestamp = t;
      return true;
   }
   std::vector<pvgpu_entry> e;
   if (!read_sparse(frame, e, timestamp, err)) return false;
   std::memset(out, 0, sizeof(float) * (size_t)n);
   for (const pvgpu_entry &x : e) out[x.index] = x.value;
   return true;
}

}  // namespace pvhost
