/*
 * rtacx -- C ABI of the GB300 receiver-side reduction for rtac_simulation.
 *
 * The reference computes a sonar ping from ray-cast echo samples in three
 * steps, all behind SensorInstance::compute_output():
 *   sort(samples)          src/Receiver.cu:9-42 (thrust::sort by travel)
 *   binner_.compute(...)   include/rtac_simulation/Binner.h:96-102,
 *                          src/Binner.cu:24-136 (keys, segments, windows)
 *   do_reduce(...)         src/SensorInstance2D.cu:44-119 (2D),
 *                          src/SensorInstance1D.cu:35-89 (1D)
 * This library replaces those three steps. Plain pointers and sizes only;
 * device pointers are caller-owned (as SensorInstance owns receivedSamples_
 * and the ping) and are never permuted: unlike the reference, the caller's
 * sample buffer is left in its original order. Every call is stream-ordered
 * on the caller's stream (a cudaStream_t passed as void*, NULL = legacy
 * default stream) and returns without a device-wide synchronisation.
 * Errors are status codes, never exceptions or device traps; the message of
 * the last failure is available from rtacx_last_error().
 *
 * Sample layouts (include/rtac_simulation/Sample.h:101-161):
 *   RTACX_SAMPLE_1D  SimSample1D {float re, im, travel}            12 bytes
 *   RTACX_SAMPLE_2D  SimSample2D {float re, im, travel, bearing}   16 bytes
 * A null sample has travel = -1 and value 0 (Sample.h:122-127, 155-160).
 * Outputs are complex64 (interleaved float re, im): 1D ping [range_count],
 * 2D ping row-major [range_count][bearing_count], i.e. cell (r, b) at
 * r * bearing_count + b as out(blockIdx.y = r, blockIdx.x = b) in
 * src/SensorInstance2D.cu:81.
 */
#ifndef RTACX_H
#define RTACX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rtacx_ctx rtacx_ctx;
typedef int rtacx_status;

#define RTACX_OK                    0
#define RTACX_ERR_INVALID_ARGUMENT  1  /* bad pointer, size or configuration */
#define RTACX_ERR_NOT_CONFIGURED    2  /* call needs rtacx_configure_* first  */
#define RTACX_ERR_CUDA              3  /* a CUDA runtime call failed          */
#define RTACX_ERR_OUT_OF_MEMORY     4  /* scratch allocation failed           */
#define RTACX_ERR_DEVICE            5  /* device error word set by a kernel   */
#define RTACX_ERR_UNSUPPORTED       6  /* size or mode beyond this build      */

/* Key of a sample outside [min - margin, max + margin] (Binner::Key::OutOfRange,
 * include/rtac_simulation/Binner.h:27). */
#define RTACX_KEY_OUT_OF_RANGE 0xFFFFFFFFu

#define RTACX_SAMPLE_1D 1
#define RTACX_SAMPLE_2D 2

/* rtacx_sensor_1d.flags: use the literal 1D PSF scaling of the reference,
 * scaling.x = 1.0f / duration * c (src/SensorInstance1D.cu:30), instead of
 * the evident intent 1 / (duration * c) that the 2D path uses. */
#define RTACX_FLAG_1D_LITERAL_SCALING 1u

/* rtacx_sensor_2d.flags: evaluate the PSF as the reference does, by a
 * linear-filtered texture fetch (src/SensorInstance2D.cu:14-15, 20-42,
 * include/rtac_simulation/ReductionKernel.h:63-69) on the GPU's texture
 * unit, whose bilinear weights are fixed point (1/256): rtacx_reduce then
 * reproduces the reference's 2D pings to float round-off. Without the flag
 * the PSF uses exact bilinear weights (the FP64 rendition the plain form
 * meets at 1e-5), which differ from the reference's pings by up to a few
 * 1e-3 relative L2. The flag keeps range-only bins (one contiguous sample
 * run per output row, as the reference's bin views) and a slower gather
 * (one texture fetch per sample and output cell). The batched and the
 * allocation-free entry points do not take it (RTACX_ERR_UNSUPPORTED). */
#define RTACX_FLAG_TEXTURE_PSF 2u
/* On a 1D sensor (rtacx_sensor_1d.flags) RTACX_FLAG_TEXTURE_PSF fetches the
 * pulse as the reference's 1D kernel does (tex1D of a one-row float2 texture,
 * linear filter, normalized coordinates; src/SensorInstance1D.cu:15-33,
 * include/rtac_simulation/ReductionKernel.h:44-55). The reference sets
 * neither filter nor address mode there, so both are rtac_base defaults that
 * are not vendored: border addressing is taken, or clamp addressing with
 * RTACX_FLAG_TEXTURE_CLAMP as well. Measured on the reference's own kernel:
 * with border addressing the fetch blends the pulse row with the zero row
 * beyond it and returns half the pulse; with clamp addressing it returns the
 * pulse, extended by its edge taps outside the table. rtacx_reduce then
 * reproduces the reference's 1D pings in either mode to float round-off.
 * Without the flags the 1D pulse is the exact linear interpolation of the
 * table, zero outside it (the evident intent). */
#define RTACX_FLAG_TEXTURE_CLAMP 4u
/* rtacx_sensor_2d.flags: gather with the FP32 CUDA-core kernel instead of the
 * tensor-core one. By default a 2D ping's gather (output tiles of 64 ranges x
 * 128 bearings) forms its sample-by-PSF outer products on the tcgen05 tensor
 * cores from TF32 operands split in hi + lo parts (three products, FP32
 * accumulation: the same accuracy as the FP32 path, the float additions in
 * another order). */
#define RTACX_FLAG_SIMT_GATHER 8u

/* 1D echosounder (SensorInstance1D, include/rtac_simulation/SensorInstance1D.h). */
typedef struct {
    float range_min;        /* ranges_: Linspace<float>(min, max, count)     */
    float range_max;
    uint32_t range_count;
    float sound_celerity;   /* soundCelerity_ (m/s)                           */
    float pulse_duration;   /* waveform_->duration() (s)                      */
    float margin;           /* Binner margin (m); the reference uses c*duration
                               (src/SensorInstance.cu:32)                    */
    const float* pulse;     /* host, pulse_len complex taps (Waveform table)  */
    uint32_t pulse_len;
    uint32_t flags;
} rtacx_sensor_1d;

/* 2D imaging sonar (SensorInstance2D, include/rtac_simulation/SensorInstance2D.h). */
typedef struct {
    float range_min;
    float range_max;
    uint32_t range_count;
    float sound_celerity;
    float pulse_duration;
    float margin;
    const float* pulse;     /* host, pulse_len complex taps: texture height    */
    uint32_t pulse_len;
    const float* beam;      /* host, beam_len real taps (BeamDirectivity):
                               texture width (src/SensorInstance2D.cu:20-33)  */
    uint32_t beam_len;
    float beam_span;        /* BeamDirectivity::span() (rad)                  */
    const float* bearings;  /* host, bearing_count output bearings (rad),
                               SensorInfo2D::bearings()                       */
    uint32_t bearing_count;
    uint32_t flags;
} rtacx_sensor_2d;

/* Create a context bound to CUDA device `device`. Replaces the per-sensor
 * state the reference keeps in SensorInstance (Binner, PSF texture, bins_). */
rtacx_status rtacx_create(rtacx_ctx** ctx, int device);
void rtacx_destroy(rtacx_ctx* ctx);
const char* rtacx_last_error(const rtacx_ctx* ctx);
const char* rtacx_version(void);

/* Configure for a 1D / 2D sensor. Replaces SensorInstance::set_ranges
 * (src/SensorInstance.cu:23-34: Binner::reconfigure + generate_psf_data,
 * src/SensorInstance1D.cu:15-25, src/SensorInstance2D.cu:20-33) and the PSF
 * scalings of kernel() (src/SensorInstance1D.cu:27-33,
 * src/SensorInstance2D.cu:35-42). Tables are copied; synchronous. */
rtacx_status rtacx_configure_1d(rtacx_ctx* ctx, const rtacx_sensor_1d* sensor);
rtacx_status rtacx_configure_2d(rtacx_ctx* ctx, const rtacx_sensor_2d* sensor);

/* Pre-size the scratch for up to max_samples samples so that later calls
 * allocate nothing (e.g. before stream capture). Synchronous. */
rtacx_status rtacx_reserve(rtacx_ctx* ctx, uint64_t max_samples);

/* Sort + bin only (parity seam). Replaces sort() (src/Receiver.cu:9-42) and
 * Binner::compute (include/rtac_simulation/Binner.h:96-102). Every output is
 * optional (NULL to skip) and device-resident:
 *   keys      [n]                 range key of each input sample, input order
 *                                  (Binner::Key, Binner.h:47-53)
 *   segments  [range_count][2]    {start, end} of each range bin in the
 *                                  reference's travel-sorted order
 *                                  (binIndexes_, src/Binner.cu:51-80)
 *   windows   [range_count][2]    {offset, size} of each output bin's sample
 *                                  view in that order (bins_, src/Binner.cu:82-136)
 *   counts    [range_count]       samples per range bin
 *   oor       [2] (uint64)        samples out of range below / above
 * Positions are those of the reference's sorted array; this library's own
 * sorted scratch groups samples by (range bin, bearing bin) instead. */
rtacx_status rtacx_bin(rtacx_ctx* ctx, const void* samples, uint64_t n, int sample_kind,
                       uint32_t* keys, uint32_t* segments, uint32_t* windows,
                       uint32_t* counts, uint64_t* oor, void* stream);

/* Full ping: sort, bin and sparse PSF reduction into `out` (device,
 * complex64). Replaces SensorInstance1D::reduce_samples
 * (include/rtac_simulation/SensorInstance1D.h:63-69) and
 * SensorInstance2D::fill_ping / reduce_samples
 * (include/rtac_simulation/SensorInstance2D.h:66-93). `samples` must match
 * the configured sensor (12-byte records for 1D, 16-byte records for 2D) and
 * be 4-byte aligned; `out` must be 8-byte aligned (whole complex64 cells are
 * stored): RTACX_ERR_INVALID_ARGUMENT otherwise, before any work is queued. */
rtacx_status rtacx_reduce(rtacx_ctx* ctx, const void* samples, uint64_t n,
                          float* out, void* stream);

/* Echo-sample model: the per-sample epilogue of the reference's ray
 * generator, value *= exp(i 4 pi f travel / c) / travel^2
 * (src/RayCaster.cu:37-39, 69-71), applied on the device to every sample
 * before the reduction (both forms). The reference rounds the carrier phase
 * to float (an error of up to 0.06 rad at 1.2 MHz and 120 m); here it is
 * reduced modulo one cycle in FP64. NULL or flags = 0 turns it off (the
 * default). Uses the configured sound_celerity; call after rtacx_configure_*. */
#define RTACX_ECHO_PHASE     1u   /* value *= exp(i 4 pi f travel / c) */
#define RTACX_ECHO_SPREADING 2u   /* value /= travel^2                */
/* Reduce the carrier phase with compensated float arithmetic (exact product
 * split with fmaf) instead of FP64; same accuracy (~1e-7 cycle) without the
 * FP64 pipe. */
#define RTACX_ECHO_PHASE_COMPENSATED 4u
typedef struct {
    double carrier_hz;
    uint32_t flags;
} rtacx_echo_model;
rtacx_status rtacx_set_echo_model(rtacx_ctx* ctx, const rtacx_echo_model* model);

/* Precision (tensor-core) form of a configured 2D sensor. Bins onto a grid
 * first, then contracts over bearings on the tensor cores, then filters in
 * range. Per sample s (reference range key in range, finite travel t and
 * bearing theta; float arithmetic, every operation rounded on its own):
 *   range    res = (range_max - range_min) / (range_count - 1) (the output
 *            ranges' Linspace resolution), h = 2 res (one range node every
 *            two output bins), j = floor((t - range_min) / h), alpha = (t -
 *            (range_min + j h)) / h: the value goes to nodes j and j + 1
 *            with weights 1 - alpha and alpha;
 *   bearing  a uniform grid of grid_count bearings from grid_first to
 *            grid_last, step = (grid_last - grid_first) / (grid_count - 1),
 *            q = clamp(floor((theta - grid_first) / step), 0, grid_count - 2),
 *            w = clamp((theta - (grid_first + q step)) / step, 0, 1): grid
 *            bearings q and q + 1 with weights 1 - w and w
 *            (divisions as products with the float reciprocals);
 *   G[j][q] += v_s times the product of the two weights (four cells);
 *   out(r, b) = sum_t taps[r % 2][t] sum_q G[r / 2 + t - tap_center][q]
 *            D[q][b], D the dense complex [grid_count][bearing_count]
 *            directivity (D[q][b]: response of beam b to grid bearing q); a
 *            row whose reference window (do_make_bins rule,
 *            src/Binner.cu:90-102, on the keyed non-empty range bins) is
 *            empty is zero.
 * Each sample costs two 16-byte vector reductions: the grid is stored by
 * bearing interval (the shares of its two bearings side by side). The
 * contraction runs in BF16 with three split products (hi*hi + hi*lo +
 * lo*hi) and FP32 accumulation on tcgen05 tensor cores; the rest is FP32.
 * NULL tables are derived from the 2D sensor: taps[p][t] the least-squares
 * (L2) projection of the pulse response pulse(x - p res) (texture-equivalent
 * lerp, seen from a node) onto the hat functions of the nodes (the weight of
 * node offset t - tap_center), and D[.][b] the least-squares projection of
 * beam(theta - theta_b) onto the bearing grid's hat functions (the
 * coefficients whose linear interpolation between grid bearings is closest
 * in mean square to the per-sample response). On the 512-bearing
 * 2^24-sample benchmark ping the derived model is within 6e-3 to 7e-3
 * relative L2 of the per-sample PSF. grid_count 0 selects four grid bearings
 * per output bearing (rounded up to a multiple of 32); grid_first ==
 * grid_last selects the first and last table bearings. Samples outside the
 * grid's bearings take its end bearing. */
typedef struct {
    const float* directivity;   /* host complex [grid_count][bearing_count] or NULL */
    const float* range_taps;    /* host complex [2][tap_count] (even, odd rows) or NULL */
    uint32_t tap_count;         /* taps per output-row parity (<= 1024)            */
    uint32_t tap_center;        /* index of node offset 0                          */
    uint32_t flags;             /* 0 or RTACX_PRECISION_* below                     */
    uint32_t grid_count;        /* bearing grid size (even, <= 16384), 0: default   */
    float grid_first;           /* first and last grid bearing (rad)                */
    float grid_last;
} rtacx_precision_desc;
/* Contract in FP16 instead of BF16: each row of the filtered grid and each
 * column of the directivity is scaled by a power of two to [2^14, 2^15)
 * before the fp16 [hi | hi | lo] x [hi | lo | hi] split (11-bit halves,
 * products exact in the FP32 accumulator) and the scales are undone exactly
 * in the GEMM epilogue. */
#define RTACX_PRECISION_FP16_ROWSCALE 1u
/* Contention relief for clustered scenes (a strong target concentrating many
 * samples in few range bins): a strided subsample of each ping (1/128 of the
 * samples, or of the first 2^21-record chunk of rtacx_reduce_precision_host)
 * finds the densest interval of 128 range nodes (256 output bins); if it holds at least a
 * tenth of the samples and four times its uniform share, those rows are
 * accumulated into eight replicas (chosen by CTA and warp), added back into
 * the grid before the contraction, so vector reductions to the same cells no
 * longer serialise. Same result up to the order of float additions. */
#define RTACX_PRECISION_HOT_RANGE 2u
rtacx_status rtacx_configure_precision(rtacx_ctx* ctx, const rtacx_precision_desc* desc);
rtacx_status rtacx_reduce_precision(rtacx_ctx* ctx, const void* samples, uint64_t n,
                                    float* out, void* stream);

/* The precision form from HOST memory, the end-to-end call of a host-side
 * caller (the reference fills `samples()` from host vectors before
 * SensorInstance::compute_output(), include/rtac_simulation/SensorInstance.h:67,
 * and reads `output()` back). `samples` holds n host records (pinned memory
 * lets the copies overlap); they are copied to the device in chunks of
 * RTACX_STREAM_CHUNK records through two staging buffers on an internal copy
 * stream, each copy overlapping the accumulation of the previous chunk, and
 * the ping is copied to `out` (host, range_count x bearing_count complex64).
 * Stream-ordered on `stream`: `out` is valid once the stream completes. */
#define RTACX_STREAM_CHUNK (1u << 21)
rtacx_status rtacx_reduce_precision_host(rtacx_ctx* ctx, const void* samples, uint64_t n,
                                         float* out, void* stream);

/* Echo-sample epilogue (no counterpart in this path of the reference: it
 * restates the ray generator's and receiver's per-hit arithmetic,
 * src/RayCaster.cu:49-81 and include/rtac_simulation/Receiver.h:51-60, so
 * that sample buffers can be produced on the device from hit lists without
 * OptiX). Per hit: distance < 1e-4 gives a null sample (value 0, travel -1);
 * otherwise value *= exp(i 4 pi f d / c) / d^2 (per `flags`, carrier phase
 * reduced in FP64), localDir = R^T dir, value *= directivity(atan2(ly, lx) /
 * pi, atan2(lz, lx) / pi) (float table, normalized coordinates, bilinear,
 * mirror addressing, include/rtac_simulation/Directivity.h:30-34), bearing =
 * atan2(-ly, lx) (Sample.h:150). Writes 12-byte or 16-byte sample records for
 * the configured 1D / 2D sensor (its sound_celerity). */
typedef struct {
    float re, im;            /* complex value reaching the receiver          */
    float distance;          /* travel (m)                                   */
    float dir_x, dir_y, dir_z; /* ray direction, world frame                 */
} rtacx_echo;
typedef struct {
    float rotation[9];       /* receiver pose rotation R, row-major           */
    const float* directivity;/* host [height][width] table, NULL = uniform 1  */
    uint32_t directivity_width;
    uint32_t directivity_height;
    double carrier_hz;
    uint32_t flags;          /* RTACX_ECHO_PHASE | RTACX_ECHO_SPREADING        */
} rtacx_receiver;
rtacx_status rtacx_configure_receiver(rtacx_ctx* ctx, const rtacx_receiver* receiver);
rtacx_status rtacx_make_samples(rtacx_ctx* ctx, const rtacx_echo* hits, uint64_t n, void* samples, void* stream);

/* Receiver directivity tables of Directivity::rectangle_antenna and
 * Directivity::disk_antenna (src/Directivity.cpp:59-101, 109-166), built on the
 * device. params: rectangle {width, height, wavelength, baffle, oversampling},
 * disk {diameter, wavelength, baffle, oversampling} (baffle 0 none, 1
 * single-sided; lengths in one unit). Writes the table size; with out != NULL
 * also the row-major [height][width] float table (device). */
#define RTACX_DIRECTIVITY_RECTANGLE 1
#define RTACX_DIRECTIVITY_DISK      2
rtacx_status rtacx_directivity_table(int kind, const float* params, float* out, uint32_t* width,
                                     uint32_t* height, void* stream);

/* Rasterised echo samples: the OpenGL ray caster's vertex and fragment
 * shader arithmetic (src/RayCasterGL.cpp:5-63) and its framebuffer readback
 * into SimSample2D records (src/SimulationGL.cu:105-171), on CUDA, without a
 * graphics stack. The mesh is drawn with a depth test (nearest fragment, the
 * first triangle on ties); every pixel gets (a cos phase, a sin phase, range,
 * bearing) with a = reflected / range^2 / cos(bearing) / cos(elevation),
 * phase = range * 4 pi f / c + pi / 2 (reduced in FP64), or zeros where no
 * triangle covers it; rows bottom-up (glReadPixels order), width x height
 * records. Matrices are row-major (p' = M p). Triangles with a vertex behind
 * the eye or outside a +/-64 NDC guard band are skipped (GL would clip them).
 * Scratch grows on demand inside the context. */
typedef struct {
    const float* vertices;        /* device [n_vertices][3], world frame   */
    const float* normals;         /* device [n_vertices][3]                */
    const uint32_t* triangles;    /* device [n_triangles][3] vertex indices */
    uint32_t n_vertices;
    uint32_t n_triangles;
} rtacx_mesh;
typedef struct {
    float world_to_local[16];     /* worldToLocal (receiver frame)         */
    float world_to_screen[16];    /* worldToScreen (clip space)            */
    float origin[3];              /* sensor position, world frame          */
    uint32_t width;
    uint32_t height;
    double carrier_hz;            /* the reference's shader uses 1.2e6     */
    float sound_celerity;         /* ... and 1500                          */
} rtacx_raster_view;
rtacx_status rtacx_rasterize(rtacx_ctx* ctx, const rtacx_mesh* mesh, const rtacx_raster_view* view,
                             float* samples, void* stream);

/* Batched plain form: many pings from heterogeneous sensors (each bound to
 * its own configured 1D or 2D context, whose scratch it uses) in one CUDA
 * graph holding ONE kernel: a cooperative persistent launch (every CTA
 * resident) that zeroes, counts, scans, windows, scatters and gathers every
 * ping, taking work from atomic queues (gather tiles heaviest first) and
 * separating the phases with grid barriers whose waits are bounded (about
 * 1 s): a CTA that gives up sets the batch status word and stops, and so
 * does every other CTA at the next barrier (rtacx_batch_status reports it;
 * the pings are then incomplete; the next run starts clean). With
 * RTACX_BATCH_STAGED the graph holds one launch per binning stage and a
 * persistent gather instead. The reference has no batching (one
 * SensorInstance::compute_output per ping, each kernel followed by a device
 * sync). rtacx_batch_plan binds the pings (samples, counts, outputs are baked
 * into the graph: re-plan when any of them changes) and, with
 * RTACX_BATCH_AUTOTUNE, times every candidate gather tile shape x samples
 * per binning chunk on this batch and keeps the fastest. rtacx_batch_run
 * replays the graph on `stream`. Results equal rtacx_reduce's per ping with
 * RTACX_FLAG_SIMT_GATHER (the batch gathers on the CUDA cores), and the
 * default tensor-core gather's to float round-off. */
typedef struct rtacx_batch rtacx_batch;
typedef struct {
    rtacx_ctx* ctx;          /* configured context, one per ping          */
    const void* samples;     /* device samples matching the context       */
    uint64_t n;              /* sample count, >= 1                        */
    float* out;              /* device ping (complex64)                   */
} rtacx_ping_desc;
#define RTACX_BATCH_AUTOTUNE 1u
#define RTACX_BATCH_STAGED   2u
rtacx_status rtacx_batch_create(rtacx_batch** batch, int device);
void rtacx_batch_destroy(rtacx_batch* batch);
const char* rtacx_batch_last_error(const rtacx_batch* batch);
rtacx_status rtacx_batch_plan(rtacx_batch* batch, const rtacx_ping_desc* pings, uint32_t count, uint32_t flags);
rtacx_status rtacx_batch_run(rtacx_batch* batch, void* stream);
/* Wait for `stream` and report the batch status word (RTACX_ERR_DEVICE if a
 * grid-barrier wait of a run expired since the last check; clears it). The
 * per-ping device error words stay on the pings' contexts
 * (rtacx_stream_status). */
rtacx_status rtacx_batch_status(rtacx_batch* batch, void* stream);
/* Number of kernel nodes in the planned graph (1 for the fused form). */
rtacx_status rtacx_batch_graph_kernels(const rtacx_batch* batch, uint32_t* kernels);
/* Diagnostic for the failure path (no counterpart in the reference), taken
 * into account by the next rtacx_batch_plan: the fused kernel's grid barriers
 * wait for `extra_arrivals` (0 or 1) more CTAs than the launch has, so with 1
 * the first barrier never completes and every CTA gives up after `wait_ms`
 * (1..10000; default 1000) and returns. */
rtacx_status rtacx_diag_batch_barrier(rtacx_batch* batch, uint32_t extra_arrivals, uint32_t wait_ms);
/* The plan's choice: gather tile rows x bearings, samples per binning CTA,
 * and the autotuned batch time in ms (0 without autotuning). */
rtacx_status rtacx_batch_tuning(const rtacx_batch* batch, uint32_t* tile_rows, uint32_t* tile_bearings,
                                uint32_t* samples_per_cta, float* tuned_ms);

/* Wait for `stream` and report the device error word of this context
 * (RTACX_ERR_DEVICE if a kernel flagged an error since the last check).
 * Clears the word. */
rtacx_status rtacx_stream_status(rtacx_ctx* ctx, void* stream);

/* Stage tracing (no counterpart in the reference, which has no timers):
 * when enabled, rtacx_reduce records a CUDA event pair around each stage on
 * the caller's stream. rtacx_stage_times waits for the last traced call and
 * writes up to `max` stage durations in milliseconds (0 for stages the last
 * call did not run): for rtacx_reduce count, reset of the bin totals, bin
 * scan, scatter, windows, reduce; for rtacx_reduce_precision accumulate,
 * operand split, range filter, tensor-core GEMM, (unused), and the zeroing
 * of the grid before the accumulation. Returns the number of stages written
 * (negative on error). */
#define RTACX_STAGE_COUNT 6
rtacx_status rtacx_set_tracing(rtacx_ctx* ctx, int enable);

/* Diagnostic for the failure path (no counterpart in the reference): the
 * staged precision accumulation of this context skips the bulk copy of
 * sample stage `stage` (1024 records each; 0xFFFFFFFF: none, the default).
 * The CTA waiting for it gives up after about one second, sets a bit in the
 * device error word, waits (bounded) for its other copies and stops; the
 * ping is then incomplete and rtacx_stream_status returns RTACX_ERR_DEVICE.
 * The context stays usable: the next ping clears its grid. */
rtacx_status rtacx_diag_drop_accumulation_stage(rtacx_ctx* ctx, uint32_t stage);

/* Diagnostic (no counterpart in the reference): copies the first
 * min(max_records, capacity) records of the context's sorted scratch, as
 * left by the last rtacx_bin / rtacx_reduce queued on `stream`, into
 * `records` (device or pinned host memory, 16 bytes per record): float4
 * {re, im, travel, bearing} (bearing 0 for 1D sensors; the value after the
 * echo model when one is set). The first n - (out-of-range count) records
 * are the binned samples, each once, grouped by composite key (range bin x
 * bearing sub-bins + bearing sub-bin) in ascending order, in any order
 * inside a group. */
rtacx_status rtacx_diag_sorted(rtacx_ctx* ctx, float* records, uint64_t max_records, void* stream);
int rtacx_stage_times(rtacx_ctx* ctx, float* ms, int max);

/* Diagnostic: synchronous C = A * B^T on the tensor cores (the GEMM of the
 * precision form). A [M][K], B [N][K] bf16, C [M][N] fp32, row-major,
 * device pointers 16-byte aligned; M % 128 == 0, N % 128 == 0, K % 64 == 0.
 * No counterpart in the reference. */
rtacx_status rtacx_gemm_bf16_tn(const void* A, const void* B, float* C, int M, int N, int K, void* stream);

/* Allocation-free ping. No counterpart in the reference: it exists for
 * callers that cannot call cudaMalloc -- sensor loops running under an
 * allocation ban (no driver allocation locks in a real-time step) or
 * processes whose device memory belongs to another allocator. It runs the
 * same kernels as rtacx_reduce without a context: the sensor (a
 * rtacx_sensor_1d* or rtacx_sensor_2d* matching sample_kind, host tables) is
 * uploaded on every call into one fixed file-scope device array that also
 * holds all scratch (about 6.6 MB, kept by every GPU that loads the library
 * until exit). Runs on the current device and on `stream`; no cudaMalloc,
 * cudaFree or other allocating call. Sizes above the limits below return
 * RTACX_ERR_UNSUPPORTED. The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress): make it before any stream capture.
 * All calls share the array, so calls whose GPU work overlaps (other streams,
 * other threads) race: serialise them. `samples` must be 4-byte and `out`
 * 8-byte aligned (RTACX_ERR_INVALID_ARGUMENT otherwise). Status codes only
 * (no context, so no rtacx_last_error message); the kernels' device error
 * word is not read back, so a consistency error on the device (which an
 * overlapping call can cause) is not reported by the status. */
#define RTACX_NOALLOC_MAX_SAMPLES  (1u << 18)
#define RTACX_NOALLOC_MAX_RANGES   4096u
#define RTACX_NOALLOC_MAX_BEARINGS 1024u
#define RTACX_NOALLOC_MAX_PULSE    4096u
#define RTACX_NOALLOC_MAX_BEAM     8192u
rtacx_status rtacx_reduce_noalloc(int sample_kind, const void* sensor, const void* samples,
                                  uint64_t n, float* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* RTACX_H */
