/* fbp.h — C ABI of the GB300 reconstruction library (libfbp.so).
 *
 * Plain pointers and sizes only.  Every device pointer argument is a CUDA
 * device address on the context's device; `stream` is a cudaStream_t passed
 * as void* (NULL = legacy default stream).  Calls are asynchronous on
 * `stream` unless stated otherwise and never throw: each returns an
 * fbp_status, and fbp_last_error() gives the message of the last failure on
 * the calling thread.
 *
 * Each entry point names the reference interface it replaces
 * (paths relative to the reference's FasterBackprojection/ directory).
 * A call that takes a context runs on the context's device and leaves the
 * calling thread's current device as it found it.
 */
#ifndef FBP_H
#define FBP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FBP_ABI_VERSION 1

typedef enum {
    FBP_OK = 0,
    FBP_ERR_INVALID_ARG = 1, /* null pointer, zero or inconsistent size, unknown enum */
    FBP_ERR_OOM = 2,         /* device or host allocation failed */
    FBP_ERR_CUDA = 3,        /* a CUDA runtime call or kernel launch failed */
    FBP_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up (status word set) */
    FBP_ERR_UNSUPPORTED = 5, /* valid but not implemented for these arguments */
    FBP_ERR_DEVICE = 6,      /* a kernel reported an internal check failure */
    FBP_ERR_IO = 7,          /* file could not be read or written */
    FBP_ERR_INTERNAL = 8     /* unexpected host-side failure inside the library (message in fbp_last_error) */
} fbp_status;

/* Storage type of a transient cube. */
typedef enum { FBP_F32 = 0, FBP_BF16 = 1, FBP_F16 = 2 } fbp_dtype;

/* Order of a confocal cube with L scan points and T bins.
 *   FBP_LAYOUT_TIME_MAJOR: cube[t*L + l] — what the reference kernels index
 *                          (transient_utils.cuh:6-9).
 *   FBP_LAYOUT_TIME_INNER: cube[l*T + t] — the order NLosData stores
 *                          (NLosData.cpp:241, 264) and filter_H works on.
 * Exhaustive cubes are always cube[(l*S + s)*T + t] (transient_utils.cuh:11-14). */
typedef enum { FBP_LAYOUT_TIME_MAJOR = 0, FBP_LAYOUT_TIME_INNER = 1 } fbp_layout;

typedef enum { FBP_CONFOCAL = 0, FBP_EXHAUSTIVE = 1 } fbp_capture_system;

/* Reconstruction geometry.  Same field order and packing as the reference's
 * ReconstructionInfo (GpuStructs.cuh:8-38), 148 bytes.  Distances and
 * time_step are path lengths in metres (time_step = metres per bin).
 * Voxel (vx, vy, vz) of a volume indexed [vz][vy][vx] sits at
 *   hidden_min + (vx, vz, vy) * voxel_size + voxel_size / 2
 * (transient_reconstruction.cuh:106): the outermost index drives world y. */
typedef struct {
    float sensor_position[3];
    uint32_t capture_system; /* fbp_capture_system */
    float laser_position[3];
    float time_offset;
    uint32_t num_laser_targets;
    uint32_t num_sensor_targets;
    uint32_t num_time_bins;
    float time_step;
    float hidden_min[3];
    uint32_t discard_first_last_bounces; /* 0: add |l-laser| + |s-sensor| to each path */
    float hidden_max[3];
    float hidden_size[3];
    float voxel_size[3];
    float wall_min[3];
    float wall_size[3];
    float wall_normal[3];
    uint32_t voxel_res[3]; /* (Vx, Vy, Vz) */
} fbp_recon_info;

typedef struct fbp_context fbp_context;

/* ---- library / context ------------------------------------------------- */

const char* fbp_version(void);
/* Message of the last failed call on this thread ("" if none). */
const char* fbp_last_error(void);

/* Replaces CudaContext (CudaContext.cpp:6-58) and the reference's global
 * __constant__ state (GpuStructs.cu:4-16): a context owns per-call geometry
 * tables and grow-only scratch on one device, so calls are reentrant across
 * contexts.  One context must not be used from two host threads at once. */
fbp_status fbp_create(fbp_context** ctx, int device);
fbp_status fbp_destroy(fbp_context* ctx);
/* Read and clear the context's device status word (set by bounded waits and
 * internal checks).  Synchronises `stream`. */
fbp_status fbp_check_device_status(fbp_context* ctx, void* stream);
/* Number of kernels this context launched since creation (instrumentation). */
uint64_t fbp_kernel_launch_count(const fbp_context* ctx);

/* How the voxel gathers compute the per-pair weight safeRCP(dist^2)
 * (math.cuh:23-29, transient_reconstruction.cuh:131), which the reference
 * evaluates with one fast-math reciprocal per (voxel, scan point) pair.
 *   FBP_WEIGHTS_BATCHED   (default) groups of voxels of one thread share one
 *                         reciprocal (Montgomery's simultaneous inversion):
 *                         each weight within ~4 ulp of the reference's, the
 *                         bins still bit for bit; volumes within 1e-6 relative
 *                         L2 of the reference-weight result.
 *   FBP_WEIGHTS_REFERENCE every weight is the reference's own reciprocal, so a
 *                         single-scan-point volume equals the reference kernel's
 *                         bit for bit (slower: one reciprocal per pair).
 * Applies to fbp_backproject_confocal, _slab, _exhaustive, fbp_mis_backproject
 * (unbiased modes) and batches created afterwards.  No counterpart in the
 * reference (an option of this library). */
typedef enum { FBP_WEIGHTS_BATCHED = 0, FBP_WEIGHTS_REFERENCE = 1 } fbp_weight_mode;
fbp_status fbp_set_weight_mode(fbp_context* ctx, int mode);
fbp_status fbp_get_weight_mode(const fbp_context* ctx, int* mode);

/* ---- backprojection ------------------------------------------------------ */

/* Confocal voxel backprojection.  Replaces Laser::reconstructAABBConfocal
 * (Laser.cu:482-498) + backprojectConfocalVoxel (transient_reconstruction.cuh:93-136).
 * volume[Vx*Vy*vz + vy*Vx + vx] = sum over scan points l of
 *     I(l, bin) * safeRCP(dist^2)   for I > 1e-5 and 0 <= bin < T,
 *     dist = 2|l - p| - time_offset (+ bounce terms), bin = int(dist / time_step).
 * The volume is overwritten (the reference adds into a zeroed buffer).
 * Bin indices follow the reference's FP32 fast-math expression bit for bit;
 * sums are FP32 per block of scan points, compensated (Kahan) across blocks,
 * in a fixed order, so results are reproducible run to run.
 * cube: L*T elements of `dtype` in `layout`; laser_xyz: L*3 floats. */
fbp_status fbp_backproject_confocal(fbp_context* ctx, const fbp_recon_info* info, const void* cube, int dtype,
                                    int layout, const float* laser_xyz, float* volume, void* stream);

/* Exhaustive (laser x SPAD) voxel backprojection.  Replaces
 * Laser::reconstructAABBExhaustive (Laser.cu:500-516) + backprojectExhaustiveVoxel
 * (transient_reconstruction.cuh:138-166), with the pair split l = ls / S,
 * s = ls % S (the reference splits by L, which equals this only when L == S).
 * cube: (l*S + s)*T + t; laser_xyz: L*3; sensor_xyz: S*3. */
fbp_status fbp_backproject_exhaustive(fbp_context* ctx, const fbp_recon_info* info, const void* cube, int dtype,
                                      const float* laser_xyz, const float* sensor_xyz, float* volume, void* stream);

/* Depth-plane backprojection (unweighted).  Replaces Laser::reconstructDepthConfocal /
 * reconstructDepthExhaustive (Laser.cu:379-480) + backprojectConfocal /
 * backprojectExhaustive (transient_reconstruction.cuh:41-91).
 * activation[c*D + d] for c < L: test point laser_xyz[c] + wall_normal * float(depths[d]).
 * `layout` applies to confocal cubes only; sensor_xyz may be NULL for confocal. */
fbp_status fbp_backproject_depths(fbp_context* ctx, const fbp_recon_info* info, const void* cube, int dtype,
                                  int layout, const float* laser_xyz, const float* sensor_xyz,
                                  const double* depths, uint32_t num_depths, float* activation, void* stream);

/* Transient images: the output step of the depth-plane reconstruction
 * (Laser::reconstructDepthConfocal / Exhaustive, Laser.cu:409-424, 461-476) and
 * of NLosData::saveImages (NLosData.cpp:161-180), for num_planes planes at once.
 * Pixel idx (row-major, idx < width*height) of plane p is
 * data[p*plane_stride + idx*pixel_stride] (device): pixel_stride D, plane_stride 1
 * for the depth planes of an [L][D] activation; 1 and width*height for
 * contiguous slices.  Each plane becomes TransientImage::save's image
 * (TransientImage.cpp:46-64): grey RGBA8 clamp(uint(v*255), 0, 255), rows flipped
 * (Image.h:160-178), bilinearly resized to out_width x out_height when that
 * differs (Image.h:45-66, 92-138), in the reference's FP32 expression order.
 * rgba: device [num_planes][out_height][out_width][4], PNG row order.  normalize
 * != 0 divides each plane by max(0, its maximum) first (the reference divides
 * the first width*height floats of its pointer: the same plane for contiguous
 * slices).  Sizes 1..65535; a resized image is at least 2 x 2. */
fbp_status fbp_transient_images(fbp_context* ctx, const float* data, uint32_t width, uint32_t height,
                                uint32_t num_planes, uint64_t pixel_stride, uint64_t plane_stride, uint32_t out_width,
                                uint32_t out_height, int normalize, uint8_t* rgba, void* stream);

/* PNG file (8-bit RGBA) of a host image, rows top first; replaces the SOIL2
 * SOIL_save_image call of TransientImage::save (TransientImage.cpp:63).  Host function. */
fbp_status fbp_write_png(const char* path, const uint8_t* rgba, uint32_t width, uint32_t height);

/* fbp_transient_images, then "<prefix>transient_<p>.png" for every plane
 * (Laser.cu:416-424, NLosData.cpp:172-178).  Synchronises the stream. */
fbp_status fbp_save_transient_images(fbp_context* ctx, const float* data, uint32_t width, uint32_t height,
                                     uint32_t num_planes, uint64_t pixel_stride, uint64_t plane_stride,
                                     uint32_t out_width, uint32_t out_height, int normalize, const char* prefix,
                                     void* stream);

/* Laser::linearSpace (Laser.cu:69-78) and the depth set reconstructShapeDepths
 * uses (Laser.cu:365-377): out[i] = min + i*(max-min)/n.  Host function. */
fbp_status fbp_linear_space(double min_value, double max_value, int n, double* out);

/* Diagnostic: the time-bin index the backprojection uses for each
 * (voxel, scan point) pair — bins[i*L + l] for voxel linear index voxel_idx[i]
 * (confocal), bins[(i*L + l)*S + s] (exhaustive); -1 where the bin is outside
 * [0, T).  Same FP32 expression as the gathers; used by the parity tests. */
fbp_status fbp_debug_confocal_bins(fbp_context* ctx, const fbp_recon_info* info, const float* laser_xyz,
                                   const int64_t* voxel_idx, uint64_t num_voxels, int32_t* bins, void* stream);
fbp_status fbp_debug_exhaustive_bins(fbp_context* ctx, const fbp_recon_info* info, const float* laser_xyz,
                                     const float* sensor_xyz, const int64_t* voxel_idx, uint64_t num_voxels,
                                     int32_t* bins, void* stream);
/* Diagnostic: the path length dist = 2|l - p| - time_offset (+ bounce terms)
 * of each confocal (voxel, scan point) pair in the gathers' FP32 expression
 * (transient_reconstruction.cuh:127-130), paths[i*L + l], and in consts[0..1]
 * (device) rcp.approx(time_step) and half the voxel diagonal: with these a CPU
 * replays the voxel-scattering walk's bins (transient_reconstruction.cuh:112-126)
 * exactly.  Used by the parity tests. */
fbp_status fbp_debug_confocal_paths(fbp_context* ctx, const fbp_recon_info* info, const float* laser_xyz,
                                    const int64_t* voxel_idx, uint64_t num_voxels, float* paths, float* consts,
                                    void* stream);

/* ---- sampled (MIS) backprojection ----------------------------------------- */

typedef enum {
    FBP_MIS_UNIFORM = 0,   /* unbiased, scan points uniform per voxel tile */
    FBP_MIS_SPATIAL = 1,   /* unbiased, p(l) proportional to scan point l's total intensity */
    FBP_MIS_LEARNED = 2,   /* unbiased, whole scan clusters drawn per tile (systematic sampling) from a
                              per-tile cluster distribution (fbp_mlp_forward), uniform when none is given */
    FBP_MIS_REFERENCE = 3, /* the reference kernel's one-sample balance-heuristic MIS */
    FBP_MIS_REFERENCE_SCATTER = 4 /* FBP_MIS_REFERENCE as the reference's ACCUMULATE_VOXEL_SCATTERING build
                                     computes it (transient_reconstruction.cuh:235-250): each sample adds every
                                     bin of dist -/+ half the voxel diagonal, stepped by time_step + 1e-5, until a
                                     bin leaves [0, T); time_step must exceed 1e-4 m */
} fbp_mis_proposal;

typedef struct {
    int proposal;            /* fbp_mis_proposal */
    uint32_t samples;        /* per voxel tile: scan points (UNIFORM, SPATIAL) or clusters (LEARNED, <= 256);
                                per voxel (REFERENCE; 0 = L/4) */
    uint64_t seed;           /* unbiased modes: counter-based RNG seed */
    const float* noise;      /* REFERENCE: device uniform buffer (NULL: numVoxels from std::mt19937) */
    uint64_t noise_size;
    const float* tile_cluster_cdf; /* LEARNED: device [tiles][G] inclusive CDF over scan clusters (NULL: uniform),
                                      tiles in fbp_mis_tile_grid order (x fastest) */
    uint32_t cluster_side;   /* LEARNED: clusters are cluster_side^2 blocks of the scan grid */
    uint32_t scan_side;      /* LEARNED: scan grid side (L = scan_side^2, l = iz*side + ix) */
    uint32_t cv_side;        /* LEARNED: 0, or the side of the scan-point blocks summed into the control
                                variate (divides cluster_side and scan_side): the estimate is then the full
                                backprojection of the block-summed capture plus the sampled clusters'
                                real-minus-block-summed contributions (still unbiased) */
} fbp_mis_params;

/* Sampled confocal backprojection.  Replaces Laser::reconstructAABBConfocalMIS
 * (Laser.cu:526-611), buildAliasTables (:253-315) and backprojectConfocalVoxelMIS
 * (transient_reconstruction.cuh:194-260).  The unbiased modes estimate the full
 * backprojection: every voxel tile draws `samples` scan points from the proposal
 * and weights each by 1/(samples * p(l)).  REFERENCE keeps the reference's
 * arithmetic and RNG (biased), with its spatial CDF built from the capture and
 * samples summed in order per voxel. */
fbp_status fbp_mis_backproject(fbp_context* ctx, const fbp_recon_info* info, const void* cube, int dtype,
                               int layout, const float* laser_xyz, const fbp_mis_params* params, float* volume,
                               void* stream);
/* Diagnostic: the REFERENCE mode's proposal tables for this capture, copied
 * to host arrays of L entries (normalised spatial CDF, alias, probability). */
fbp_status fbp_mis_reference_tables(fbp_context* ctx, const fbp_recon_info* info, const void* cube, int dtype,
                                    int layout, float* spatial_cdf, uint32_t* alias, float* prob, void* stream);
/* Voxel tiles of the gather / MIS sampling: tiles[0..2] along (vx, vy, vz). */
fbp_status fbp_mis_tile_grid(const fbp_recon_info* info, uint32_t tiles[3]);

/* The reference's ACCUMULATE_VOXEL_SCATTERING build of backprojectConfocalVoxel
 * (transient_reconstruction.cuh:112-126, a compile-time option there): each
 * (voxel, scan point) pair adds I(bin) * safeRCP(dist^2) for every bin of
 * d = max(0, dist - e), d += timeStep + 1e-5 while d < dist + e, with e half
 * the voxel diagonal, in the reference's FP32 arithmetic and order.
 * time_step must exceed 1e-4 m. */
fbp_status fbp_backproject_confocal_scatter(fbp_context* ctx, const fbp_recon_info* info, const void* cube, int dtype,
                                            int layout, const float* laser_xyz, float* volume, void* stream);

/* Scatter-form backprojection: the reference's rasterised ellipsoid splat
 * (DrawEllipsoids.cpp:12-114, 332-440, shaders backprojection-vs/fs.glsl, an
 * OpenGL path) on CUDA.  Every (scan point, bin < max_bins) with intensity
 * above FLT_EPSILON is a hemisphere towards -y of radius
 * (bin * time_step + time_offset [- bounces]) / 2 around the scan point,
 * sampled at a grid_w x grid_h grid of pixel centres over the volume's x / z
 * extent; each sample adds the intensity to the voxel it falls in (FP32
 * atomics, like imageAtomicAdd).  max_bins 0 = all bins (the reference uses
 * 700).  The volume is overwritten. */
fbp_status fbp_splat_backproject(fbp_context* ctx, const fbp_recon_info* info, const void* cube, int dtype, int layout,
                                 const float* laser_xyz, uint32_t max_bins, uint32_t grid_w, uint32_t grid_h,
                                 float* volume, void* stream);

/* ---- depth-slab partition across ranks ------------------------------------ */

/* No counterpart in the reference (it runs on one GPU).  Voxels are
 * independent, so ranks reconstruct contiguous ranges of depth slices of the
 * same capture with no collective on the data path; the slabs are gathered
 * afterwards.
 * fbp_plan_slabs: z_bounds[0..nranks] (nranks + 1 entries), slab r is
 * [z_bounds[r], z_bounds[r+1]); boundaries are multiples of 16 (the gather's
 * tile depth) except the last (= voxel_res[2]); balanced by tile rows. */
fbp_status fbp_plan_slabs(const fbp_recon_info* info, uint32_t nranks, uint32_t* z_bounds);
/* Bins [*bin_lo, *bin_hi] that any voxel of slices [z_begin, z_end) can reach
 * from any scan point (FP64 box distances, 2 bins of margin, clamped to
 * [0, T-1]; *bin_lo > *bin_hi if none).  laser_xyz: HOST array, L*3.  A rank
 * may copy only these bins of the capture to its GPU (zeros elsewhere). */
fbp_status fbp_slab_bin_window(const fbp_recon_info* info, const float* laser_xyz, uint32_t z_begin, uint32_t z_end,
                               uint32_t* bin_lo, uint32_t* bin_hi);
/* fbp_backproject_confocal restricted to slices [z_begin, z_end) into
 * volume_slab[z_end - z_begin][Vy][Vx]; with z_begin a multiple of 16 the
 * slab is bitwise the same rows of the full volume. */
fbp_status fbp_backproject_confocal_slab(fbp_context* ctx, const fbp_recon_info* info, const void* cube, int dtype,
                                         int layout, const float* laser_xyz, uint32_t z_begin, uint32_t z_end,
                                         float* volume_slab, void* stream);

/* ---- learned MIS proposal (MLP on the tensor cores) ----------------------- */

/* No counterpart in the reference: its MIS proposal is the spatial alias table
 * over scan points (Laser.cu:253-315).  Here a 19 -> 64 -> 64 -> 64 -> 1 MLP
 * (GELU, BF16 weights and operands on tcgen05 tensor cores, FP32 accumulation
 * in TMEM) scores every (voxel tile, scan cluster) pair; FBP_MIS_LEARNED
 * draws whole clusters from the per-tile distribution it yields.
 * Clusters are cluster_side^2 blocks of the scan grid (scan_side^2 points,
 * l = iz*scan_side + ix), at most 1024 per capture.  Tiles are the gather's
 * 8 x 16 x 16-voxel tiles in fbp_mis_tile_grid order (x fastest).
 * Feature rows hold FBP_MLP_FEATURES floats (19 inputs + 1 pad). */
#define FBP_MLP_FEATURES 20

typedef struct fbp_mlp fbp_mlp;

uint32_t fbp_mlp_num_params(void);
/* Random initialisation (uniform +-1/sqrt(fan_in), zero biases) from `seed`. */
fbp_status fbp_mlp_create(fbp_context* ctx, uint64_t seed, fbp_mlp** out);
fbp_status fbp_mlp_destroy(fbp_mlp* mlp);
/* Flat FP32 parameter vector: W1[64][32] (inputs 19..31 zero), b1[64],
 * W2[64][64], b2, W3[64][64], b3, w4[64], b4.  set_params resets Adam. */
fbp_status fbp_mlp_get_params(const fbp_mlp* mlp, float* host, uint32_t n);
fbp_status fbp_mlp_set_params(fbp_mlp* mlp, const float* host, uint32_t n);
fbp_status fbp_mlp_tile_count(const fbp_recon_info* info, uint32_t* ntiles);
/* Feature rows [ntiles][G][FBP_MLP_FEATURES] (device) of the listed tiles
 * (device list; NULL = every tile, ntiles ignored). */
fbp_status fbp_mlp_features(fbp_context* ctx, const fbp_recon_info* info, const void* cube, int dtype, int layout,
                            const float* laser_xyz, uint32_t cluster_side, uint32_t scan_side, const uint32_t* tiles,
                            uint32_t ntiles, float* features, void* stream);
/* Training targets [ntiles][G] (device): per tile, q_c proportional to
 * sqrt(sum over the tile's voxels of F_vc^2), F_vc = cluster c's exact
 * contribution (the reference kernel's arithmetic) to voxel v. */
fbp_status fbp_mlp_labels(fbp_context* ctx, const fbp_recon_info* info, const void* cube, int dtype, int layout,
                          const float* laser_xyz, uint32_t cluster_side, uint32_t scan_side, const uint32_t* tiles,
                          uint32_t ntiles, float* labels, void* stream);
/* Forward pass: logits [ntiles][G] and/or the per-tile inclusive CDF
 * [ntiles][G] of (1 - defensive) * softmax + defensive / G (either may be NULL). */
fbp_status fbp_mlp_forward(fbp_context* ctx, const fbp_mlp* mlp, const float* features, uint32_t ntiles, uint32_t G,
                           float* logits, float defensive, float* tile_cdf, void* stream);
/* Gradient of the mean softmax cross-entropy over the minibatch rows idx
 * (device, nbatch entries indexing features/labels) into grad_loss (device,
 * fbp_mlp_num_params() + 1 floats: the gradient, then the loss). */
fbp_status fbp_mlp_gradients(fbp_context* ctx, const fbp_mlp* mlp, const float* features, const float* labels,
                             const uint32_t* idx, uint32_t nbatch, uint32_t G, float* grad_loss, void* stream);
/* One Adam step (beta 0.9 / 0.999) on that gradient; the minibatch loss is
 * copied to `loss` (device, may be NULL). */
fbp_status fbp_mlp_train_step(fbp_context* ctx, fbp_mlp* mlp, const float* features, const float* labels,
                              const uint32_t* idx, uint32_t nbatch, uint32_t G, float lr, float* loss, void* stream);

/* ---- batched reconstruction ---------------------------------------------- */

/* One confocal capture of a batch (all captures of a batch share `dtype`). */
typedef struct {
    fbp_recon_info info;    /* geometry, by value */
    const void* cube;       /* device, L*T elements in `layout` */
    int dtype;              /* fbp_dtype */
    int layout;             /* fbp_layout */
    const float* laser_xyz; /* device, L*3 */
    float* volume;          /* device, [Vz][Vy][Vx], overwritten by each run */
} fbp_capture_desc;

typedef struct fbp_batch fbp_batch;

/* Batched form of fbp_backproject_confocal for many captures of uneven sizes
 * (the reference reconstructs one capture per run, Laser.cu:40-67).  Plans
 * every capture once and allocates the batch's own device buffers; the
 * descriptors (device pointers included) are copied and must stay valid. */
fbp_status fbp_batch_create(fbp_context* ctx, uint32_t n, const fbp_capture_desc* captures, fbp_batch** out);
/* Re-reads every capture's cube and writes every volume: one persistent
 * launch over all (capture, voxel tile) work items, largest captures first.
 * use_graph != 0: the launches are captured into a CUDA graph on the first
 * call and replayed afterwards (needs a non-default stream). */
fbp_status fbp_batch_run(fbp_batch* batch, int use_graph, void* stream);
/* Times every voxel-tile shape on this batch and keeps the fastest (index in
 * *chosen).  Synchronises `stream`; drops a captured graph. */
fbp_status fbp_batch_autotune(fbp_batch* batch, void* stream, int* chosen);
/* Selects tile shape `config` (0..3) explicitly: 16 x 16 x 16, 8 x 16 x 16,
 * 8 x 32 x 16 or 4 x 32 x 16 voxels (x, y, depth); 0 is the single-capture
 * gather's tile. */
fbp_status fbp_batch_set_config(fbp_batch* batch, int config, void* stream);
fbp_status fbp_batch_destroy(fbp_batch* batch);

/* ---- post-processing ------------------------------------------------------ */

typedef enum { FBP_FILTER_NONE = 0, FBP_FILTER_LAPLACIAN = 1, FBP_FILTER_LOG = 2, FBP_FILTER_LOG_FFT = 3 } fbp_filter;

/* PostprocessingFilters::compute (PostprocessingFilters.h:5-39) for
 * None / Laplacian / LoG / LoGFFT.  in and out are [nz][ny][nx] floats and
 * must not alias (the reference writes a new buffer and swaps, :29-31).
 * NONE copies in to out.  LOG_FFT keeps the reference's unnormalised inverse
 * (scale nx*ny*nz) and requires power-of-two sizes. */
fbp_status fbp_postfilter(fbp_context* ctx, int kind, int kernel_size, float sigma, const float* in, float* out,
                          uint32_t nx, uint32_t ny, uint32_t nz, void* stream);

/* The LoG weights the reference builds on the host
 * (LoG::calculateLaplacianKernel, PostprocessingFilters.cu:102-175). Host function;
 * w receives size^3 floats. */
fbp_status fbp_log_weights(int size, float sigma, float* w);

/* Laser::normalizeMatrix (Laser.cu:317-339): v = (v - min) * safeRCP(max - min),
 * in place, min/max reduced on the device. */
fbp_status fbp_normalize_minmax(fbp_context* ctx, float* v, uint64_t n, void* stream);

/* fbp_normalize_minmax without allocating: no counterpart in the reference.
 * For callers that cannot let a library call cudaMalloc — an acquisition
 * loop that reserves the whole device memory budget up front, or a host
 * application whose own allocator owns every device byte.  Needs no
 * context; runs on the current device, and v must be device memory of that
 * device (FBP_ERR_INVALID_ARG otherwise).  Its scratch is a fixed 8 KiB array
 * inside libfbp on each device, so n is limited to 2^30 elements
 * (FBP_ERR_UNSUPPORTED beyond).  Each call looks up that array's device
 * address; the first call on a device also loads the library's device code
 * there, so make that first call before any stream capture.  A CUDA error
 * already pending when the call starts is returned as FBP_ERR_CUDA without
 * launching anything (and is not cleared).  Calls that overlap on the GPU
 * share the array and race; order them (one stream, or events). */
fbp_status fbp_normalize_minmax_noalloc(float* v, uint64_t n, void* stream);

/* ---- temporal filter ------------------------------------------------------ */

typedef enum { FBP_BORDER_ZERO = 0, FBP_BORDER_EDGE = 1 } fbp_border;

/* Laser::filter_H_cuda (Laser.cu:128-240) on device data, in place:
 * data[i*T + t] for i < num_series.  Band-pass with the complex
 * Gaussian-windowed wave of mean wavelength wl_mean (same units as
 * delta_t), sigma = wl_sigma (0 selects wl_mean / sqrt(2)), zero or edge
 * padding by t6sigma - 1, unnormalised inverse, real part kept — computed
 * as the equivalent real correlation instead of padded FFTs. */
fbp_status fbp_filter_h(fbp_context* ctx, float* data, uint64_t num_series, uint32_t num_bins, float delta_t,
                        float wl_mean, float wl_sigma, int border, void* stream);

/* ---- light-cone transform ------------------------------------------------ */

/* Radiometric grid of the LCT.  python/lct.py:134-136 builds grid_z with
 * np.tile(..., (1, N, N)).reshape(M, N, N), so voxel (z, y, x) is scaled by
 * linspace(0, 1, M)[(z*N + y) % M]; FBP_LCT_GRID_DEPTH scales by [z] instead,
 * the per-depth grid the surrounding comments describe. */
typedef enum { FBP_LCT_GRID_REFERENCE = 0, FBP_LCT_GRID_DEPTH = 1 } fbp_lct_grid;

/* What the LCT keeps of the complex volume after the inverse resampling.
 *   FBP_LCT_OUTPUT_CLAMPED_REAL  max(real(vol), 0)   (python/lct.py:154)
 *   FBP_LCT_OUTPUT_MAGNITUDE     abs(vol)            (python/lct_2.py:154)
 * python/lct_2.py is lct.py with this output, FBP_LCT_GRID_DEPTH's radiometry
 * (lct_2.py:103) and the PSF normalised by its column at (U, U) instead of
 * (U-1, U-1) (lct_2.py:202 against lct.py:333); that last difference cancels,
 * since the PSF is then normalised by its L2 norm. */
typedef enum { FBP_LCT_OUTPUT_CLAMPED_REAL = 0, FBP_LCT_OUTPUT_MAGNITUDE = 1 } fbp_lct_output;

typedef struct {
    float width;      /* half-width of the scanned wall area in metres (lct.py `width`) */
    float bin_length; /* metres of path per bin (c * bin resolution) */
    float snr;        /* Wiener filter SNR (lct.py: 0.8) */
    int diffuse;      /* 1: grid_z^4 radiometry (diffuse), 0: grid_z^2 */
    int grid_mode;    /* fbp_lct_grid */
    int output;       /* fbp_lct_output */
} fbp_lct_params;

/* Confocal LCT reconstruction (python/lct.py:97-211 without the file loading,
 * downsampling and z_trim; the C++ LCT::reconstructAABB, LCT.cpp:16-18, is an
 * empty stub in the reference).  data: N x N scan points x M bins, either
 * FBP_LAYOUT_TIME_MAJOR [M][N][N] or FBP_LAYOUT_TIME_INNER [N][N][M];
 * volume: [M][N][N] floats (depth, y, x).  N, M powers of two <= 2048.
 * The PSF's Wiener filter and the resampling operator are cached in the
 * context for the last (N, M, width/range, snr). */
fbp_status fbp_lct(fbp_context* ctx, const float* data, int layout, uint32_t N, uint32_t M,
                   const fbp_lct_params* params, float* volume, void* stream);

/* ---- end to end (host buffers) ---------------------------------------------- */

typedef struct {
    int use_fourier_filter;   /* TransientParameters::_useFourierFilter (default 1) */
    int postfilter;           /* fbp_filter (default NONE) */
    int kernel_size;          /* default 5 */
    float sigma;              /* default 1 */
    int normalize;            /* min-max normalise the result (the reference always does) */
} fbp_shape_params;

/* Laser::reconstructShape for the AABB mode (Laser.cu:40-67, 341-363) from
 * HOST buffers: optional filter_H on the time-innermost cube, upload,
 * confocal or exhaustive backprojection, post-filter, min-max normalise,
 * download into volume_host ([Vz][Vy][Vx] floats).  cube_host is
 * time-innermost (NLosData::_data order) in `dtype`; for F32 and
 * use_fourier_filter the filter runs on the device copy, the host cube is not
 * modified.  Synchronous. */
fbp_status fbp_reconstruct_shape_host(fbp_context* ctx, const fbp_recon_info* info, const void* cube_host,
                                      int dtype, const float* laser_xyz_host, const float* sensor_xyz_host,
                                      const fbp_shape_params* params, float* volume_host, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* FBP_H */
