/*
 * satgb.h -- C ABI of libsatgb.so, a GB300 (sm_103a) summed-area-table
 * (integral image) library.
 *
 * A drop-in for the three algorithm entry points of pengdada/SAT
 * (integralImage/*.cu).  In the reference each one is a host driver that
 * launches two kernels on caller-visible device buffers:
 *
 *   ScanRow-BRLT  (BlockScan)      BlockScan::Test / blockScan x2   ScanRow-BRLT.cu:182-255, kernel :24-180
 *   BRLT-ScanRow  (SerialScan)     SerielScan::Test / serielScan x2 BRLT-Scan.cu:192-266,    kernel :15-127
 *   ScanRowColumn (IncreamentScan) IncrementScan::Test / ScanX,ScanY ScanRowColumn.cu:424-499, kernels :16-268
 *
 * Here each entry point computes the same result -- the inclusive 2-D prefix
 * sum out(y,x) = sum_{j<=y, i<=x} in(j,i) of a row-major width x height image
 * -- with ONE launch of a single-pass tiled kernel (decoupled look-back in both
 * tile directions), reading every input element once and writing every output
 * element once.
 *
 * Conventions (kept from the reference):
 *   - buffers are caller-owned DEVICE pointers;
 *   - pitches are in ELEMENTS of the buffer's own type (GpuData::DataPitch,
 *     cudaLib.cuh:178-180), pitch >= width;
 *   - dtype codes are the reference's DataType enum (integralImage.h:22-32);
 *   - scan_type is the reference's SCAN enum (integralImage.h:34-37).
 *     Kogge-Stone and Ladner-Fischer give identical integer results; for
 *     floating point this library's summation tree is its own and floats are
 *     checked against an FP64 oracle, so scan_type is validated and recorded
 *     but does not change the arithmetic.
 * Added over the reference (which reports no errors: CUDA_CHECK_ERROR is an
 * empty macro, cudaLib.cuh:21-22): every call returns a satgb_status; calls
 * are asynchronous on the given stream (a cudaStream_t passed as void*, NULL
 * = legacy default stream); device-side failures (a look-back wait that
 * exceeded its time limit) are reported by satgb_stream_check().
 *
 * Integer outputs wrap modulo 2^32 exactly like the reference's CPU integral
 * image (IntegralImageSerial, integralImage.h:105-124).
 *
 * Scratch: the look-back status words live in a per-stream workspace that the
 * library allocates on first use (and grows when a larger image arrives) and
 * frees in satgb_release().  A call on an image of 1-byte inputs of at least
 * 2^22 pixels whose rows are not 16-byte aligned (base or pitch) also copies
 * its input into padded rows in that workspace (one extra launch; the
 * workspace grows by about the input's size).  Calls on distinct streams may
 * run concurrently; calls on one stream are ordered by the stream.
 */
#ifndef SATGB_H
#define SATGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SATGB_VERSION 100 /* 1.0.0 */

typedef enum {
  SATGB_OK = 0,
  SATGB_ERR_INVALID_ARG = 1,       /* null pointer, width/height <= 0, pitch < width, bad enum */
  SATGB_ERR_UNSUPPORTED_TYPES = 2, /* dtype pair (or mode) not offered */
  SATGB_ERR_MISALIGNED = 3,        /* pointer not aligned to its element size */
  SATGB_ERR_OVERFLOW = 4,          /* sizes whose byte extent does not fit in int64 */
  SATGB_ERR_ALLOC = 5,             /* workspace allocation failed */
  SATGB_ERR_CUDA = 6,              /* a CUDA runtime call failed (see satgb_last_error_string) */
  SATGB_ERR_TIMEOUT = 7,           /* a device-side look-back wait exceeded its limit */
  SATGB_ERR_NOT_FOUND = 8          /* no such plan / symbol / tuning entry */
} satgb_status;

/* The reference's DataType enum, integralImage.h:22-32.  u16/i16 are listed
 * there but never dispatched; they are rejected here too. */
typedef enum {
  SATGB_U8 = 0,
  SATGB_I8 = 1,
  SATGB_U16 = 2,
  SATGB_I16 = 3,
  SATGB_U32 = 4,
  SATGB_I32 = 5,
  SATGB_F32 = 6,
  SATGB_F64 = 7
} satgb_dtype;

/* The reference's SCAN enum, integralImage.h:34-37. */
typedef enum { SATGB_SCAN_KOGGE_STONE = 0, SATGB_SCAN_LF = 1 } satgb_scan_type;

typedef enum {
  SATGB_MODE_PLAIN = 0,       /* arithmetic in the output type */
  SATGB_MODE_COMPENSATED = 1  /* f32 outputs only: two-sum compensated carries */
} satgb_mode;

typedef enum {
  SATGB_FORWARD = 0, /* out(y,x) = sum_{j<=y, i<=x} in(j,i)   (the SAT) */
  SATGB_REVERSE = 1  /* out(y,x) = sum_{j>=y, i>=x} in(j,i)   (suffix SAT; the SAT's adjoint) */
} satgb_direction;

typedef void* satgb_stream; /* a cudaStream_t */

/* ------------------------------------------------------------------------- */
/* The three drop-in entry points.                                            */
/* Type pairs (in_t -> out_t), as dispatched by the reference's host drivers  */
/* (ScanRow-BRLT.cu:274-376, BRLT-Scan.cu:287-390, ScanRowColumn.cu:518-621): */
/*   u8 -> u32, f32, f64      i8 -> i32, f32, f64      i32 -> i32, f64        */
/*   f32 -> f32, f64          f64 -> f64                                      */
/* plus u32 -> u32 (the reference's TDst -> TDst second-pass instantiation).  */
/* ------------------------------------------------------------------------- */

/* Replaces BlockScan::Test<TSrc,TDst,SCAN_TYPE> (ScanRow-BRLT.cu:182-255):
 * its two blockScan launches (:225-226) over devA -> devTmp -> devB. */
satgb_status satgb_scanrow_brlt(satgb_dtype in_t, satgb_dtype out_t, int scan_type,
                                const void* d_in, int64_t in_pitch,
                                void* d_out, int64_t out_pitch,
                                int64_t width, int64_t height, satgb_stream stream);

/* Replaces SerielScan::Test<TSrc,TDst,SCAN_TYPE> (BRLT-Scan.cu:192-266):
 * its two serielScan launches (:237-238). */
satgb_status satgb_brlt_scanrow(satgb_dtype in_t, satgb_dtype out_t, int scan_type,
                                const void* d_in, int64_t in_pitch,
                                void* d_out, int64_t out_pitch,
                                int64_t width, int64_t height, satgb_stream stream);

/* Replaces IncrementScan::Test<TSrc,TDst,SCAN_TYPE> (ScanRowColumn.cu:424-499):
 * its ScanX + ScanY launches (:475-476). */
satgb_status satgb_scanrowcolumn(satgb_dtype in_t, satgb_dtype out_t, int scan_type,
                                 const void* d_in, int64_t in_pitch,
                                 void* d_out, int64_t out_pitch,
                                 int64_t width, int64_t height, satgb_stream stream);

/* ------------------------------------------------------------------------- */
/* Extended single-image call: compensated f32 and the reverse (suffix) SAT.  */
/* No reference counterpart (the reference has neither).                      */
/* ------------------------------------------------------------------------- */
typedef struct {
  satgb_dtype in_t, out_t;
  int mode;      /* satgb_mode */
  int direction; /* satgb_direction */
  const void* d_in;
  int64_t in_pitch;
  void* d_out;
  int64_t out_pitch;
  int64_t width, height;
} satgb_sat_desc;

satgb_status satgb_sat_ex(const satgb_sat_desc* desc, satgb_stream stream);

/* Row-only and column-only scans, the two halves of ScanRowColumn as separate
 * operations: out(y,x) = sum_{i<=x} in(y,i) (IncrementScanX::ScanX,
 * integralImage/IncrementScanX.cu:12-113, and the first launch of
 * ScanRowColumn.cu:475) and out(y,x) = sum_{j<=y} in(j,x) (IncrementScanY::ScanY,
 * integralImage/IncrementScanY.cu:10-126).  Same type pairs, pitches and
 * conventions as the SAT entry points. */
satgb_status satgb_scan_rows(satgb_dtype in_t, satgb_dtype out_t, const void* d_in, int64_t in_pitch,
                             void* d_out, int64_t out_pitch, int64_t width, int64_t height, satgb_stream stream);
satgb_status satgb_scan_cols(satgb_dtype in_t, satgb_dtype out_t, const void* d_in, int64_t in_pitch,
                             void* d_out, int64_t out_pitch, int64_t width, int64_t height, satgb_stream stream);

/* Row scan with transposed output, out(x, y) = sum_{i<=x} in(y, i): the input
 * is width x height (pitch in_pitch), the output height x width, i.e. width
 * rows of height elements (pitch out_pitch >= height).  Replaces the
 * reference's SerielScan::TestX (integralImage/BRLT-Scan.cu:128-190), one
 * serielScan launch whose output is IntegralImageAllRow transposed.  Same
 * type pairs as the scans; input and output must not overlap. */
satgb_status satgb_scan_rows_transposed(satgb_dtype in_t, satgb_dtype out_t, const void* d_in, int64_t in_pitch,
                                        void* d_out, int64_t out_pitch, int64_t width, int64_t height,
                                        satgb_stream stream);

/* The same SAT for a stack of n_planes equally sized images (e.g. the N*C
 * planes of an N x C x H x W tensor), plane p starting at d_in + p *
 * in_plane_stride and d_out + p * out_plane_stride (elements); each plane gets
 * its own SAT, all in one launch.  No reference counterpart. */
satgb_status satgb_sat_planes(const satgb_sat_desc* desc, int64_t n_planes, int64_t in_plane_stride,
                              int64_t out_plane_stride, satgb_stream stream);

/* ------------------------------------------------------------------------- */
/* Box filters from a SAT (f32), the main use of a summed-area table.  No     */
/* reference counterpart.  For radius r the box mean at (y,x) is the mean of  */
/* the input over rows [y-r, y+r] and columns [x-r, x+r] clipped to the       */
/* image, read from the inclusive SAT S of the input by four corners:         */
/*   (S(yb,xb) - S(ya-1,xb) - S(yb,xa-1) + S(ya-1,xa-1)) / area.              */
/* Up to four radii are filtered in one pass over n_planes planes.            */
/* Limits: width <= 2^30, height <= 65535 * 32, n_planes <= 65535; f32 only.  */
/* Radii >= 0; a radius above max(width, height) - 1 filters like that radius */
/* (its window already covers the whole image).                               */
/* ------------------------------------------------------------------------- */
#define SATGB_MAX_RADII 4
typedef struct {
  int64_t width, height, n_planes;
  void* d_sat;            /* forward: the SAT (read); backward: dL/dSAT (written) */
  int64_t sat_pitch, sat_plane_stride;
  int n_radii;            /* 1 .. SATGB_MAX_RADII */
  int radius[SATGB_MAX_RADII];
  void* d_box[SATGB_MAX_RADII]; /* forward: box means (written); backward: dL/dmeans (read) */
  int64_t box_pitch, box_plane_stride;
} satgb_box_desc;

/* Box means of every radius from the SAT. */
satgb_status satgb_box_filter_fwd(const satgb_box_desc* desc, satgb_stream stream);
/* The adjoint of satgb_box_filter_fwd: dL/dSAT from the gradients of all the
 * radii's means (the four-corner scatter, computed as a gather so it is
 * deterministic).  d_sat is overwritten. */
satgb_status satgb_box_filter_bwd(const satgb_box_desc* desc, satgb_stream stream);
/* The gradient of the box means with respect to the image the SAT was taken
 * of, dL/dx = reverse SAT of dL/dSAT, in one call and without scratch memory:
 * dL/dSAT is gathered into d_dx, then d_dx is reverse-summed in place (two
 * tile launches and the edge launch of satgb_box_filter_bwd).  desc->d_sat is
 * not used; d_dx (n_planes planes of width x height, pitch and plane stride in
 * elements) is written and may not overlap the gradients of the means. */
satgb_status satgb_box_filter_bwd_x(const satgb_box_desc* desc, void* d_dx, int64_t dx_pitch,
                                    int64_t dx_plane_stride, satgb_stream stream);

/* The same single-image SAT as satgb_sat_ex, for callers that cannot allocate
 * device memory: code running inside an allocator or memory-pool callback, in
 * a process whose device memory a framework has reserved up front, or in a
 * loop that must not pay for an allocation.  It has no counterpart in the
 * reference.  It calls no cudaMalloc/cudaFree: its look-back scratch is a
 * fixed 16 MiB array inside libsatgb.so that every GPU loading the library
 * holds until the process exits.  Images whose scratch does not fit are
 * rejected with SATGB_ERR_INVALID_ARG (the message gives both sizes): with
 * the tiles this entry point uses, the array holds 8,160 tiles of 128 x 128
 * pixels for plain 4-byte outputs (e.g. 10240 x 13056, or 8192 x 16256),
 * 5,433 tiles of 128 x 64 (width x height) for compensated f32 and 8,128
 * tiles of 64 x 64 for f64 outputs.  The first call on each device looks up
 * the array's device address and should come before any stream capture.  All
 * calls share the array: calls whose kernels overlap on the GPU race and give
 * wrong results.  Failures are reported like those of the other entry points
 * (status and satgb_last_error_string); device-side wait timeouts are not. */
satgb_status satgb_sat_noalloc(const satgb_sat_desc* desc, satgb_stream stream);

/* ------------------------------------------------------------------------- */
/* Batched SAT: many images of uneven sizes, one persistent launch per size   */
/* class.  No reference counterpart (the reference's drivers handle one       */
/* image).  A plan copies the image table to the device, splits the images    */
/* into two size classes (large: at least 64 tiles of 128 x 128 pixels;       */
/* small: the rest), picks a tile configuration per class (from the tuning    */
/* cache when an entry for this batch's signature exists) and captures the    */
/* classes' launches, one after the other, in one CUDA graph; exec replays    */
/* the graph on `stream`.  All images share one dtype pair, mode and          */
/* direction.  No image may write memory another image reads or writes.       */
/* Inputs whose rows TMA cannot address (base or row pitch not a multiple of  */
/* 16 bytes, rows of at least 16 bytes: e.g. packed u8 rows of odd widths)    */
/* are copied by each exec, as the graph's first launch, into rows padded to  */
/* 16 bytes in a staging buffer the plan allocates (about the size of those   */
/* inputs, through the allocator hooks when set) and frees on destroy.        */
/* ------------------------------------------------------------------------- */
typedef struct {
  const void* d_in;
  int64_t in_pitch;
  void* d_out;
  int64_t out_pitch;
  int64_t width, height;
} satgb_image;

typedef struct satgb_batch_plan_s satgb_batch_plan;

satgb_status satgb_batch_plan_create(satgb_batch_plan** plan, satgb_dtype in_t, satgb_dtype out_t,
                                     int mode, int direction, const satgb_image* images,
                                     int64_t n_images, satgb_stream stream);
satgb_status satgb_batch_plan_exec(satgb_batch_plan* plan, satgb_stream stream);
/* Launch without the graph (same kernels, same arguments). */
satgb_status satgb_batch_plan_launch(satgb_batch_plan* plan, satgb_stream stream);
satgb_status satgb_batch_plan_destroy(satgb_batch_plan* plan);
/* Tiles in the plan and the configuration index of its large class (of the
 * small class when there are no large images). */
satgb_status satgb_batch_plan_info(const satgb_batch_plan* plan, int64_t* n_tiles, int* config);
/* Per size class (index 0 large, 1 small): images, tiles and configuration
 * (-1 for an empty class).  Each pointer may be NULL or point to 2 values. */
satgb_status satgb_batch_plan_classes(const satgb_batch_plan* plan, int64_t* n_images, int64_t* n_tiles,
                                      int* configs);
/* Batch autotuner: times every tile configuration of each size class on the
 * plan's own images (launches whose results overwrite the outputs), keeps the
 * fastest, records it in the tuning cache under the batch's signature (dtype
 * pair, mode, direction, class, pixel and image counts, TMA alignment of the
 * rows, SM count; persisted in SATGB_TUNE_CACHE when set) and captures the
 * plan's graph again.  configs may be NULL or receive the 2 chosen indices. */
satgb_status satgb_batch_plan_autotune(satgb_batch_plan* plan, satgb_stream stream, int* configs);
/* Synchronises `stream` and reports (and clears) a device-side error of the
 * plan's launches, like satgb_stream_check does for single-image calls. */
satgb_status satgb_batch_plan_check(satgb_batch_plan* plan, satgb_stream stream);

/* ------------------------------------------------------------------------- */
/* Autotuner: times each tile configuration on the given buffers (which are   */
/* overwritten) and records the fastest for this dtype pair / mode / size     */
/* bucket / SM count.  Entries persist in the JSON file named by              */
/* SATGB_TUNE_CACHE when that variable is set.  best_config may be NULL.      */
/* ------------------------------------------------------------------------- */
satgb_status satgb_autotune(satgb_dtype in_t, satgb_dtype out_t, int mode,
                            const void* d_in, int64_t in_pitch, void* d_out, int64_t out_pitch,
                            int64_t width, int64_t height, satgb_stream stream, int* best_config);
/* Number of tile configurations and a printable name for one. */
int satgb_num_configs(void);
const char* satgb_config_name(int config);
/* Force a configuration for subsequent single-image calls (-1 = automatic). */
satgb_status satgb_set_config(int config);

/* ------------------------------------------------------------------------- */
/* Errors, workspace, diagnostics.                                            */
/* ------------------------------------------------------------------------- */

/* Synchronises `stream`, then reports (and clears) a device-side error of the
 * calls on it since the last check: SATGB_ERR_TIMEOUT when a look-back wait
 * gave up (the results of that call are then incomplete).  A timed-out call
 * does not affect the calls after it: each launch starts with a clear error
 * word, and only the report waits here until it is read. */
satgb_status satgb_stream_check(satgb_stream stream);

/* Message for the last failing call on this host thread ("" when none). */
const char* satgb_last_error_string(void);

/* Frees every cached workspace (all streams); safe to call at any time when no
 * call is in flight. */
satgb_status satgb_release(void);

/* Pre-sizes the workspace of `stream` for images up to width x height, so that
 * a later call does not allocate (e.g. inside CUDA stream capture); this
 * includes the staging rows a large image of 1-byte inputs with unaligned
 * rows needs. */
satgb_status satgb_reserve(int64_t width, int64_t height, satgb_stream stream);

/* Allocation hook for the workspace (NULL restores cudaMalloc/cudaFree). */
typedef void* (*satgb_alloc_fn)(size_t bytes, void* ctx);
typedef void (*satgb_free_fn)(void* ptr, void* ctx);
satgb_status satgb_set_allocator(satgb_alloc_fn alloc_fn, satgb_free_fn free_fn, void* ctx);

/* Time limit of one look-back wait, in microseconds (default 2,000,000). */
satgb_status satgb_set_wait_limit_us(int64_t us);

/* Number of kernel launches this library has issued (all streams) since load:
 * lets a caller count the library's launches inside a timed region. */
int64_t satgb_launch_count(void);

/* Test hook: the tile with this global index never publishes its look-back
 * status, so the tiles that depend on it run into the wait limit and the call
 * reports SATGB_ERR_TIMEOUT.  -1 (the default) disables it. */
satgb_status satgb_debug_stall_tile(int64_t tile);

int satgb_version(void);

#ifdef __cplusplus
}
#endif
#endif /* SATGB_H */
