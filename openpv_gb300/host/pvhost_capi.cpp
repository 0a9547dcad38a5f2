// pvhost_capi.cpp -- the C API of include/pvhost.h over pvhost::Column.
#include "pvhost.h"

#include "column.hpp"
#include "params.hpp"

#include <cstring>
#include <new>
#include <string>

struct pvhost_column {
   pvhost::Column col;
};

namespace {
thread_local std::string g_err;
}  // namespace

namespace pvhost_capi {
pvgpu_status fail(pvgpu_status s, const std::string &msg) {
   g_err = msg;
   return s;
}
}  // namespace pvhost_capi
using pvhost_capi::fail;

namespace {

bool copy_out(const std::string &s, char *buf, size_t n) {
   if (!buf || n == 0 || s.size() + 1 > n) return false;
   std::memcpy(buf, s.c_str(), s.size() + 1);
   return true;
}

}  // namespace

extern "C" const char *pvhost_last_error(void) { return g_err.c_str(); }

extern "C" pvgpu_status pvhost_params_dump(const char *text, char *buf, size_t bufSize) {
   if (!text) return fail(PVGPU_ERR_BAD_ARG, "no params text");
   pvhost::Params p;
   std::string err;
   if (!pvhost::parse_params(text, p, err)) return fail(PVGPU_ERR_BAD_ARG, err);
   if (!copy_out(pvhost::dump_params(p), buf, bufSize)) return fail(PVGPU_ERR_BAD_ARG, "buffer too small");
   return PVGPU_OK;
}

extern "C" pvgpu_status pvhost_column_create(const char *text, pvhost_column **out) {
   if (!text || !out) return fail(PVGPU_ERR_BAD_ARG, "no params text or output");
   *out = nullptr;
   auto *c = new (std::nothrow) pvhost_column();
   if (!c) return fail(PVGPU_ERR_OOM, "out of host memory");
   std::string err;
   if (!c->col.build(text, err)) {
      delete c;
      return fail(PVGPU_ERR_BAD_ARG, err);
   }
   *out = c;
   return PVGPU_OK;
}

extern "C" pvgpu_status pvhost_column_destroy(pvhost_column *c) {
   delete c;
   return PVGPU_OK;
}

#define PVHOST_CALL(expr)                       \
   do {                                         \
      std::string err_;                         \
      pvgpu_status s_ = (expr);                 \
      if (s_ != PVGPU_OK) return fail(s_, err_); \
      return PVGPU_OK;                          \
   } while (0)

extern "C" pvgpu_status pvhost_set_weights(pvhost_column *c, const char *name, const float *w, int64_t n) {
   if (!c || !name) return fail(PVGPU_ERR_BAD_ARG, "null argument");
   PVHOST_CALL(c->col.set_weights(name, w, n, err_));
}

extern "C" pvgpu_status pvhost_set_input(pvhost_column *c, const char *name, const float *frames, int numFrames) {
   if (!c || !name) return fail(PVGPU_ERR_BAD_ARG, "null argument");
   PVHOST_CALL(c->col.set_input(name, frames, numFrames, err_));
}

extern "C" pvgpu_status pvhost_set_state(pvhost_column *c, const char *name, const float *v) {
   if (!c || !name) return fail(PVGPU_ERR_BAD_ARG, "null argument");
   PVHOST_CALL(c->col.set_state(name, v, err_));
}

extern "C" pvgpu_status pvhost_advance(pvhost_column *c, int numSteps) {
   if (!c) return fail(PVGPU_ERR_BAD_ARG, "null column");
   PVHOST_CALL(c->col.advance(numSteps, err_));
}

extern "C" pvgpu_status pvhost_read_layer(pvhost_column *c, const char *name, int which, float *host, int64_t n) {
   if (!c || !name) return fail(PVGPU_ERR_BAD_ARG, "null argument");
   PVHOST_CALL(c->col.read(name, which, host, n, err_));
}

extern "C" pvgpu_status pvhost_layer_info(pvhost_column *c, const char *name, int *out6) {
   if (!c || !name || !out6) return fail(PVGPU_ERR_BAD_ARG, "null argument");
   pvhost::Layer *L = c->col.layer(name);
   if (!L) return fail(PVGPU_ERR_BAD_ARG, std::string("no layer \"") + name + "\"");
   const int v[6] = {L->loc.nbatch, L->loc.nx, L->loc.ny, L->loc.nf, L->loc.halo.lt, L->phase};
   std::memcpy(out6, v, sizeof(v));
   return PVGPU_OK;
}

extern "C" pvgpu_status pvhost_delivery_engine(pvhost_column *c, const char *name, char *buf, size_t n) {
   if (!c || !name) return fail(PVGPU_ERR_BAD_ARG, "null argument");
   pvhost::Conn *k = c->col.conn(name);
   if (!k) return fail(PVGPU_ERR_BAD_ARG, std::string("no connection \"") + name + "\"");
   if (!copy_out(k->delivery->engine(), buf, n)) return fail(PVGPU_ERR_BAD_ARG, "buffer too small");
   return PVGPU_OK;
}

extern "C" pvgpu_status pvhost_delivery_keyword(pvhost_column *c, const char *name, char *buf, size_t n) {
   if (!c || !name) return fail(PVGPU_ERR_BAD_ARG, "null argument");
   pvhost::Conn *k = c->col.conn(name);
   if (!k) return fail(PVGPU_ERR_BAD_ARG, std::string("no connection \"") + name + "\"");
   if (!copy_out(k->delivery->keyword(), buf, n)) return fail(PVGPU_ERR_BAD_ARG, "buffer too small");
   return PVGPU_OK;
}
