/* pvhost.h -- C API of libpvhost.so, the C++ host side of the LCA hot path above libpvgpu.so.
 *
 * A column is built from the text of an OpenPV params file (HyPerCol, ImageLayer / PvpLayer
 * inputs, HyPerLayer, ANNLayer, ANNErrorLayer, HyPerLCALayer, HyPerConn, TransposeConn,
 * IdentConn) with the reference's meaning of every parameter it reads; each connection's
 * delivery is the class HyPerDeliveryCreator (delivery/HyPerDeliveryCreator.cpp:105-126) names
 * from receiveGpu / pvpatchAccumulateType / updateGSynFromPostPerspective, all of them on the
 * GPU ("...ConvolveDelivery" = the reference CPU loop's order, bit for bit).  Weights and input
 * frames come from the host (the reference reads them from files through weightInitType and
 * the input layer's inputPath).  Every call returns a pvgpu_status; pvhost_last_error() tells
 * what went wrong.  Not thread-safe per column. */
#ifndef PVHOST_H
#define PVHOST_H

#include <stddef.h>
#include <stdint.h>

#include "pvgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pvhost_column pvhost_column;

/* The message of the last failed call on this thread. */
const char *pvhost_last_error(void);

/* Parses params text (the grammar of io/parser/params.y) and writes a canonical listing (one
 * parameter per line) into buf; PVGPU_ERR_BAD_ARG with the line of the error otherwise.  No
 * GPU needed. */
pvgpu_status pvhost_params_dump(const char *paramsText, char *buf, size_t bufSize);

/* HyPerCol construction from params text: layers sized from nx, ny, nxScale, nyScale, nf;
 * halos from the margins the connections need (requiredConvolveMargin); device buffers
 * allocated; initial V per InitVType (ZeroV, ConstantV) and A = T(V) published. */
pvgpu_status pvhost_column_create(const char *paramsText, pvhost_column **out);
pvgpu_status pvhost_column_destroy(pvhost_column *c);

/* Shared weights of a HyPerConn, host FP32 [kernel][nyp][nxp][nfp]; the post weights of a
 * post-perspective delivery and the weights of every TransposeConn of it follow on the device
 * (TransposeWeights). */
pvgpu_status pvhost_set_weights(pvhost_column *c, const char *connName, const float *hostW, int64_t n);
/* Frames of an input layer, host FP32 [numFrames][nbatch][ny][nx][nf]; frame
 * ((t - 1) / displayPeriod) % numFrames is shown at timestep t (frame 0 when displayPeriod = 0). */
pvgpu_status pvhost_set_input(pvhost_column *c, const char *layerName, const float *hostFrames, int numFrames);
/* V of a non-input layer, host FP32 [nbatch][ny][nx][nf]; A = T(V) is published. */
pvgpu_status pvhost_set_state(pvhost_column *c, const char *layerName, const float *hostV);
/* HyPerCol::advanceTime numSteps times (phase order: per phase, every layer of the phase
 * receives its synaptic input, then updates and publishes); returns when the device is done. */
pvgpu_status pvhost_advance(pvhost_column *c, int numSteps);
/* V (which = 0) or the restricted activity A (which = 1) of a layer into host FP32
 * [nbatch][ny][nx][nf]; n must be that size. */
pvgpu_status pvhost_read_layer(pvhost_column *c, const char *layerName, int which, float *host, int64_t n);
/* {nbatch, nx, ny, nf, halo, phase} of a layer. */
pvgpu_status pvhost_layer_info(pvhost_column *c, const char *layerName, int *out6);
/* The delivery class a connection got, e.g. "PostsynapticPerspectiveConvolveDelivery". */
pvgpu_status pvhost_delivery_keyword(pvhost_column *c, const char *connName, char *buf, size_t bufSize);
/* Which kernel family ran the connection's last delivery: "tensor-core" (split-TF32 tcgen05),
 * "simt" (FP32 FAST kernels), "reference-order" (the Convolve keywords), "ident", or "none"
 * before the first step.  No reference counterpart (diagnostics). */
pvgpu_status pvhost_delivery_engine(pvhost_column *c, const char *connName, char *buf, size_t bufSize);


/* ---- .pvp activity files (utils/BufferUtilsPvp.hpp, io/LayerIO.cpp, io/SparseLayerIO.cpp) ----
 * Writer: header as LayerIO / SparseLayerIO::writeHeader (nBands = 0, timestamp 0), frames
 * appended, nBands rewritten after each frame.  One frame per batch element per call, in batch
 * order, as LayerOutputComponent writes them. */
typedef struct pvhost_pvp_writer pvhost_pvp_writer;
pvgpu_status pvhost_pvp_writer_open(const char *path, int nx, int ny, int nf, int sparse, pvhost_pvp_writer **out);
/* From the device: a sparse layer's SparseList (pvgpu_pvp_sparse_frames on the device, then one
 * copy of the kept entries per batch element), or a dense layer's extended activity
 * (pvgpu_pvp_dense_frames, then one copy).  Synchronises the stream. */
pvgpu_status pvhost_pvp_write_sparse_device(pvhost_pvp_writer *w, const pvgpu_loc *loc, const pvgpu_entry *entries,
                                            const int64_t *numActive, double timestamp, void *stream);
pvgpu_status pvhost_pvp_write_dense_device(pvhost_pvp_writer *w, const pvgpu_loc *loc, const float *aExt,
                                           double timestamp, void *stream);
/* From host buffers: one frame. */
pvgpu_status pvhost_pvp_write_sparse_host(pvhost_pvp_writer *w, const pvgpu_entry *entries, int32_t count,
                                          double timestamp);
pvgpu_status pvhost_pvp_write_dense_host(pvhost_pvp_writer *w, const float *restricted, double timestamp);
pvgpu_status pvhost_pvp_writer_close(pvhost_pvp_writer *w);

/* Reader: activity files of type 4 (dense), 6 (sparse values) and 2 (binary spikes). */
typedef struct pvhost_pvp_reader pvhost_pvp_reader;
pvgpu_status pvhost_pvp_reader_open(const char *path, pvhost_pvp_reader **out);
/* The 18 header ints (headerSize ... nBands) and the header timestamp; *numFrames = frames in
 * the file (from its length, as SparseLayerIO counts them). */
pvgpu_status pvhost_pvp_reader_info(pvhost_pvp_reader *r, int32_t *out18, double *timestamp, int *numFrames);
/* Frame as the restricted activity [ny][nx][nf] (n = nx*ny*nf floats). */
pvgpu_status pvhost_pvp_read_dense(pvhost_pvp_reader *r, int frame, float *host, int64_t n, double *timestamp);
/* Frame as {restricted index, value} entries (capacity entries; *count receives how many). */
pvgpu_status pvhost_pvp_read_sparse(pvhost_pvp_reader *r, int frame, pvgpu_entry *host, int64_t capacity,
                                    int32_t *count, double *timestamp);
/* Frames first .. first+nbatch-1 into a device extended activity (sparse frames scattered on the
 * device; dense frames copied into the restricted part); the halo is zeroed. */
pvgpu_status pvhost_pvp_read_to_device(pvhost_pvp_reader *r, int firstFrame, const pvgpu_loc *loc, float *aExt,
                                       void *stream);
pvgpu_status pvhost_pvp_reader_close(pvhost_pvp_reader *r);

#ifdef __cplusplus
}
#endif

#endif /* PVHOST_H */
