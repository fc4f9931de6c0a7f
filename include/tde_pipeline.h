/*
 * tde_pipeline.h -- the per-frame KinectFusion loop on one GPU.
 *
 * The reference names this layer (the `fusion` application, Makefile:1-7) but
 * does not ship it; its order follows the wrapper set of
 * common/inc/opencl_wrappers.h: bilateral filter + pyramid, vertex and normal
 * maps, coarse-to-fine ICP (10/5/4 iterations), TSDF integration, raycast of
 * the model and its map pyramid.
 *
 * GB300 design: everything stays on the device; each ICP launch starts by
 * solving the previous launch's exact totals and updating the pose in every
 * block (the frame's last launch also solves its own and publishes the FP64
 * pose), so one frame is a fixed sequence of launches with no host round
 * trip.  That sequence is
 * captured once into CUDA graphs and replayed every frame.  A frame's only
 * host traffic is the depth upload and the pose download.
 */
#ifndef TDE_PIPELINE_H
#define TDE_PIPELINE_H

#include "tde_capi.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tde_pipeline tde_pipeline;
struct tde_refiner;

typedef struct tde_pipeline_config {
    tde_intrinsics intr;         /* level-0 camera */
    tde_point3i voxels;          /* TSDF resolution */
    tde_point3f volume_size;     /* metres */
    int tsdf_format;             /* TDE_TSDF_* */
    float trunc;                 /* truncation distance, metres */
    int max_weight;              /* MAX_TSDF_WEIGHT = 128 */
    float sigma_space;           /* bilateral, pixels */
    float sigma_color;           /* bilateral and pyramid, millimetres */
    uint32_t max_depth_mm;       /* depth beyond this is invalid */
    int icp_levels;              /* 1..3 */
    int icp_iters[3];            /* per level, level 0 finest: 10, 5, 4 */
    float dist_thresh;           /* DEFAULT_DISTANCE_THRESHOLD 0.1 m */
    float angle_thresh;          /* sin(20 deg), DEFAULT_ANGLE_THRESHOLD */
    int use_graphs;              /* capture each frame's launches into CUDA graphs */
    int integrate_stats;         /* count voxels read / written by integration */
} tde_pipeline_config;

/* Frame status bits. */
#define TDE_FRAME_TRACKING_LOST 1  /* an ICP solve failed: the previous pose was kept */

/* Create a pipeline on the current device.  pose12: initial camera pose,
 * row-major R (camera -> volume frame) then t (camera centre), FP64. */
int tde_pipeline_create(const tde_pipeline_config *cfg, const double *pose12, tde_pipeline **out);
int tde_pipeline_destroy(tde_pipeline *p);
/* The pipeline's main stream (tracking, fusion, pose downloads, and every
 * call other than tde_pipeline_enqueue).  A frame's upload and preprocessing
 * run on a second, internal stream that overlaps the previous frame's
 * tracking; the main stream waits for them before the frame's tracking, so
 * work ordered after the main stream sees every enqueued frame complete. */
void *tde_pipeline_stream(tde_pipeline *p);

/* Enqueue one frame.  `depth` is cols x rows uint16 millimetres, on the host
 * (pinned for an asynchronous upload) or on the device.  When pose_out12 is
 * not NULL it must be pinned host memory of 12 doubles: the frame's pose is
 * copied there asynchronously, and *status_out (pinned int, may be NULL) gets
 * the frame status; the caller synchronises (tde_pipeline_sync) before
 * reading.  Nothing blocks. */
int tde_pipeline_enqueue(tde_pipeline *p, const uint16_t *depth, int depth_on_device, double *pose_out12,
                         int *status_out);
/* RGB-D frame: as tde_pipeline_enqueue, with rgb = cols x rows pixels of 3
 * bytes (r, g, b) registered to the depth frame (host or device as the
 * depth); required once tde_pipeline_enable_color was called, refused before.
 * The colour volume is updated right after the frame's raycast, at the model
 * surface cast from the frame's pose (tde_integrate_colors semantics). */
int tde_pipeline_enqueue_rgbd(tde_pipeline *p, const uint16_t *depth, const uint8_t *rgb, int on_device,
                              double *pose_out12, int *status_out);
/* Adds a colour volume (one tde_color per voxel, zeroed; synchronises) whose
 * weights cap at max_weight (<= 255 effective). */
int tde_pipeline_enable_color(tde_pipeline *p, int max_weight);
/* The colour volume (device; NULL without tde_pipeline_enable_color). */
int tde_pipeline_color_volume(tde_pipeline *p, tde_color **color_volume);
/* Block until all enqueued work is done. */
int tde_pipeline_sync(tde_pipeline *p);
/* Blocking convenience: enqueue, wait, return the pose (any host memory). */
int tde_pipeline_process(tde_pipeline *p, const uint16_t *depth, int depth_on_device, double *pose12,
                         int *status);

/* Current pose (synchronises). */
int tde_pipeline_pose(tde_pipeline *p, double *pose12);
/* The TSDF volume and its round buffer (device pointer, owned by the pipeline). */
int tde_pipeline_volume(tde_pipeline *p, void **volume, tde_round_buffer *rb);
/* Model maps (global frame) of pyramid level l from the last raycast. */
int tde_pipeline_model_maps(tde_pipeline *p, int level, const float **vmap, const float **nmap);
/* Current-frame filtered depth / vertex / normal maps of level l. */
int tde_pipeline_frame_maps(tde_pipeline *p, int level, const uint16_t **depth, const float **vmap,
                            const float **nmap);
/* Frames processed so far. */
int tde_pipeline_frame_count(tde_pipeline *p);

/* Live per-kernel timing: with capacity > 0, CUDA events bracket the
 * integration and raycast launches of the next `capacity` frames. */
int tde_pipeline_enable_timing(tde_pipeline *p, int capacity);
/* Milliseconds of the integration and raycast launches of the timed frames
 * (synchronises); returns the number of frames written. */
int tde_pipeline_timings(tde_pipeline *p, float *integrate_ms, float *raycast_ms, int capacity);
/* Per-stage milliseconds of the timed frames, row-major [frame][5]: input
 * preprocessing (bilateral or refiner, pyramid, vertex/normal maps, scaled
 * depth, depth tiles), ICP iterations with pose acceptance and publication
 * (pose publication alone on the first frame), integration, raycast,
 * model-map pyramid. */
int tde_pipeline_stage_timings(tde_pipeline *p, float *ms, int capacity);
/* Voxels read, voxels written and 8^3 bricks swept by integration since the
 * last reset, three counters (needs integrate_stats; synchronises). */
int tde_pipeline_integrate_stats(tde_pipeline *p, uint64_t *read_written2, int reset);
/* Number of kernel launches one tracked frame performs. */
int tde_pipeline_launches_per_frame(tde_pipeline *p);

/* Replace the volume origin bookkeeping after a cyclic shift (the caller has
 * extracted and cleaned the outgoing slab); re-captures the graphs. */
int tde_pipeline_set_round_buffer(tde_pipeline *p, const tde_round_buffer *rb);
/* Cyclic volume following the camera: the point ahead_m in front of the
 * camera (along its optical axis; half the volume keeps the volume on what
 * the camera sees) is compared with the volume centre; when it is more than
 * radius_m away along some axis, delta3 receives the shift in voxels that
 * re-centres the volume on it, else zeros. */
int tde_pipeline_shift_needed(tde_pipeline *p, float ahead_m, float radius_m, int *delta3);
/* As tde_pipeline_shift_needed for a given pose (row-major R, then t, in the
 * current volume frame) instead of the tracked one: no synchronisation, so a
 * host can decide on a shift from an earlier frame's pose (downloaded by
 * tde_pipeline_enqueue) while later frames run. */
int tde_pipeline_shift_needed_pose(tde_pipeline *p, const double *pose12, float ahead_m, float radius_m, int *delta3);

/* Shifts the volume by delta3 voxels (|delta| below the voxel count per
 * axis), host-synchronous: the slab that leaves the volume is extracted as
 * zero-crossing points (tde_extract_slice semantics and order: logical voxel
 * units of the volume before the shift; `weights` the named voxels' weights,
 * may be NULL) into host `points` up to `capacity` (the total goes to
 * *count), the slab is cleaned, the round buffer's origins advance
 * cyclically, the tracked pose moves into the new volume frame
 * (t -= delta * cell) and the model maps are cast again from it.  World
 * position of a point = origin_metric (before the shift) + point * cell. */
int tde_pipeline_shift(tde_pipeline *p, const int *delta3, tde_xyzi *points, float *weights, uint32_t capacity,
                       uint32_t *count);
/* As tde_pipeline_shift; with a colour volume, `colors` (host, may be NULL)
 * receives the points' colours and the colour slab is cleaned as well. */
int tde_pipeline_shift_ex(tde_pipeline *p, const int *delta3, tde_xyzi *points, float *weights, tde_color *colors,
                          uint32_t capacity, uint32_t *count);

/* Extract_Tsdf_Volume over the pipeline's volume, host-synchronous: every
 * zero crossing (tde_extract_tsdf_volume semantics and order: metric voxel
 * centres in the volume frame; world position = origin_metric + point) into
 * host `points` up to `capacity`, the total to *count.  `weights` (may be
 * NULL) receives the named voxels' weights; with a colour volume, `colors`
 * (may be NULL) the colours of the voxels holding the points
 * (tde_extract_color_volume).  The volume is not changed. */
int tde_pipeline_extract_volume(tde_pipeline *p, tde_xyzi *points, float *weights, tde_color *colors,
                                uint32_t capacity, uint32_t *count);

/* Generate_Image of the current model (the level-0 model maps the last
 * enqueued frame raycast) into `image` (device, cols*rows*3 bytes RGB8),
 * enqueued on the pipeline stream (tde_pipeline_sync waits for it).  `light`
 * NULL: one light at the camera centre of that frame.  Shading as
 * tde_generate_image. */
int tde_pipeline_render(tde_pipeline *p, const tde_light_source *light, uint8_t *image);

/* Checkpoint / resume.  A checkpoint holds what the next frame depends on:
 * the TSDF volume, the per-brick flags, the round buffer, the FP64 pose,
 * the frame count and, with one, the colour volume (a 272-byte header that
 * also records the intrinsics, volume edge, truncation and weight caps the
 * volume was fused with, then those buffers).  tde_pipeline_restore loads one
 * into a pipeline created with the same configuration (and
 * tde_pipeline_enable_color with the same weight cap when the checkpoint has
 * colour) and refuses any other (TDE_ERR_INVALID_ARG, nothing changed); it
 * casts the model maps again from the restored volume and pose, and the
 * frames that follow produce the same bits as they would have after the
 * checkpointed frame.  If a restore fails after its checks (a device copy
 * failed), the pipeline holds a mix of old and new state and refuses frames
 * until a later restore succeeds.  Both are host-synchronous; `buffer` is
 * host memory of tde_pipeline_checkpoint_bytes bytes. */
size_t tde_pipeline_checkpoint_bytes(tde_pipeline *p);
int tde_pipeline_checkpoint(tde_pipeline *p, void *buffer, size_t bytes);
int tde_pipeline_restore(tde_pipeline *p, const void *buffer, size_t bytes);

/* Measurement: casts the current model again from the last frame's pose
 * (into scratch maps) and counts the distinct voxel records the raycast
 * reads -- with skip_empty, as the pipeline's raycast does (skipping bricks
 * that hold no negative value), else as the reference algorithm does (every
 * sample read).  Host-synchronous; allocates scratch. */
int tde_pipeline_raycast_records(tde_pipeline *p, int skip_empty, uint64_t *records);

/* Enqueues on the pipeline's stream: the model surface of the last frame
 * (its raycast, at the pose it was tracked to) as depth along the camera axis
 * in mm, 0 where the ray found no surface -- the target of the learned
 * refiner's training pairs.  `out` is device memory of rows x cols. */
int tde_pipeline_model_depth(tde_pipeline *p, uint16_t *out);

/* Replaces the bilateral stage with the learned refiner (include/tde_refiner.h)
 * for the following frames; NULL restores the bilateral filter.  The refiner
 * must have been created for the pipeline's rows x cols and must outlive its
 * use here; refined depth feeds both ICP and integration. */
int tde_pipeline_set_refiner(tde_pipeline *p, struct tde_refiner *r);

/* Overwrite the current pose (e.g. after a shift of the volume frame). */
int tde_pipeline_set_pose(tde_pipeline *p, const double *pose12);

#ifdef __cplusplus
}
#endif
#endif
