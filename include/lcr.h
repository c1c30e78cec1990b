/*
 * liblcr -- C ABI of the GB300 (sm_103a) alignment path.
 *
 * The alignment path of LowCost3DReconstruction (scripts/alignment.sh and the
 * pcl_tools it drives, plus the depth back-projection in capture/) runs here as
 * hand-written CUDA kernels behind this plain C interface: POD arguments, host
 * pointers and sizes, no C++ types and no exceptions across the boundary.  The
 * PCL-shaped C++ facade (lcr_pcl.hpp) and the command-line tools are built on
 * these entry points; other languages bind them with their FFI.
 *
 * Ownership: the caller owns every host array it passes; the library owns
 * device clouds (lcr_cloud), which are immutable once created and are freed
 * only by lcr_cloud_free.  A cloud caches its search index on first use.
 * Threading: one lcr_ctx per host thread.  Each context owns one CUDA stream on
 * its device; calls on one context are serialised on that stream; contexts are
 * independent.  Every call returns after its results are complete unless the
 * entry point says otherwise.
 * Errors: every entry point returns an lcr_status; lcr_last_error() gives the
 * message of the last failing call on that context.  There is no CPU fallback:
 * without a usable CUDA device lcr_ctx_create fails with LCR_ERR_NO_DEVICE.
 */
#ifndef LCR_H
#define LCR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define LCR_API __attribute__((visibility("default")))
#else
#define LCR_API
#endif

typedef enum lcr_status {
  LCR_OK = 0,
  LCR_ERR_INVALID_ARG = 1,      /* bad pointer, size or parameter */
  LCR_ERR_EMPTY = 2,            /* input cloud has no (finite) points */
  LCR_ERR_NO_CORRESPONDENCES = 3, /* ICP found fewer than 3 correspondences */
  LCR_NOT_CONVERGED = 4,        /* non-fatal: result valid, criteria not met */
  LCR_ERR_CUDA = 5,             /* a CUDA runtime call failed */
  LCR_ERR_TIMEOUT = 6,          /* a bounded device wait expired */
  LCR_ERR_OOM = 7,              /* device allocation failed */
  LCR_ERR_IO = 8,               /* file could not be read or written */
  LCR_ERR_TOO_FEW_POINTS = 9,   /* k neighbours requested from a cloud with <= k points */
  LCR_ERR_NO_DEVICE = 10        /* no CUDA device */
} lcr_status;

/* Byte-compatible with pcl::PointXYZRGBNormal (48 bytes): x y z _ | nx ny nz _ |
 * b g r a (PCL's packed rgba, little-endian) curvature _ _.  A PCL cloud's
 * points.data() can be passed directly. */
typedef struct lcr_point {
  float x, y, z, pad0;
  float normal_x, normal_y, normal_z, pad1;
  uint8_t b, g, r, a;
  float curvature;
  float pad2[2];
} lcr_point;

typedef struct lcr_ctx lcr_ctx;
typedef struct lcr_cloud lcr_cloud;

/* ---------------------------------------------------------------- context */
LCR_API lcr_status lcr_ctx_create(lcr_ctx** ctx, int device);
LCR_API void lcr_ctx_destroy(lcr_ctx* ctx);
LCR_API const char* lcr_last_error(const lcr_ctx* ctx);
LCR_API const char* lcr_status_string(lcr_status s);
LCR_API lcr_status lcr_ctx_synchronize(lcr_ctx* ctx);
/* The context's cudaStream_t (as void*), for callers that order their own work
 * after the library's. */
LCR_API void* lcr_ctx_stream(lcr_ctx* ctx);
/* Number of kernels this context has launched (graph launches count each
 * kernel node executed per launch as reported by the graph's own counter). */
LCR_API uint64_t lcr_ctx_launch_count(const lcr_ctx* ctx);

/* Kernel timing (no counterpart in the reference: measurement support).  With
 * timing enabled, the launches of the listed kernels are bracketed by CUDA
 * events on the context's stream; lcr_kernel_time synchronises the stream and
 * returns the summed device time and launch count since timing was enabled.
 * lcr_kernel_timing(ctx, 1) also resets the sums.  LCR_KT_ICP_SEARCH (the
 * correspondence search of an ICP round) is timed only when the rounds run
 * from the host loop (environment LCR_ICP_GRAPH=0): inside the CUDA-graph loop
 * no event can bracket a single kernel. */
enum { LCR_KT_SOR_KNN = 0, LCR_KT_NORMALS_KNN = 1, LCR_KT_ENCODE = 2, LCR_KT_ICP_SEARCH = 3, LCR_KT_COUNT = 4 };
LCR_API lcr_status lcr_kernel_timing(lcr_ctx* ctx, int enable);
LCR_API lcr_status lcr_kernel_time(lcr_ctx* ctx, int which, double* ms, uint64_t* launches);

/* ----------------------------------------------------------------- clouds */
/* Replaces pcl::io::loadPLYFile + the PointCloud<PointXYZRGBNormal> a tool
 * holds (e.g. pcl_tools/fine_registration.cpp:94-102). */
LCR_API lcr_status lcr_cloud_upload(lcr_ctx* ctx, const lcr_point* pts, size_t n, lcr_cloud** out);
/* Same from a plain xyz array (n*3 floats); normals, rgb and curvature are 0. */
LCR_API lcr_status lcr_cloud_upload_xyz(lcr_ctx* ctx, const float* xyz, size_t n, lcr_cloud** out);
/* Same from device memory: lcr_point records already on the context's device. */
LCR_API lcr_status lcr_cloud_from_device(lcr_ctx* ctx, const void* d_pts, size_t n, lcr_cloud** out);
LCR_API size_t lcr_cloud_size(const lcr_cloud* c);
/* Copies min(n, capacity) points out; returns LCR_ERR_INVALID_ARG if capacity < n. */
LCR_API lcr_status lcr_cloud_download(lcr_ctx* ctx, const lcr_cloud* c, lcr_point* out, size_t capacity);
LCR_API void lcr_cloud_free(lcr_ctx* ctx, lcr_cloud* c);
/* The neighbour rows an lcr_normals call with LCR_NORMALS_KEEP_NEIGHBOURS kept
 * with its output cloud c: *k = the k it was called with; with host_rows
 * (32 * n words) non-NULL, row i holds in words [0, k) the indices of point
 * i's k nearest, itself included, in no particular order, and in word 31 the
 * largest squared distance among them as float bits (+inf when the cloud has
 * fewer than k finite points).  Rows of non-finite points are unspecified.
 * LCR_ERR_INVALID_ARG if c holds no rows (*k = 0). */
LCR_API lcr_status lcr_cloud_neighbours(lcr_ctx* ctx, const lcr_cloud* c, int* k, uint32_t* host_rows);
/* a followed by b (PointCloud operator+, e.g. accumulate_clouds.cpp:121-123). */
LCR_API lcr_status lcr_cloud_concat(lcr_ctx* ctx, const lcr_cloud* a, const lcr_cloud* b, lcr_cloud** out);

/* ------------------------------------------------------- back-projection */
/* Depth models: KINECT_V1 = uint16 mm through the pinhole model of
 * depth_capture.cpp:294-308; KINECT_V2 = float mm through libfreenect2's
 * registration (kinect2.h:144-201); PINHOLE_F32 = float mm through the same
 * pinhole model as V1, as super_resolution_kv2.cpp's save_ply (:25-118) writes
 * the fused Kinect v2 depth. */
enum { LCR_DEPTH_KINECT_V1 = 0, LCR_DEPTH_KINECT_V2 = 1, LCR_DEPTH_PINHOLE_F32 = 2 };

typedef struct lcr_depth_params {
  int model;                 /* LCR_DEPTH_KINECT_V1 (uint16 mm), LCR_DEPTH_KINECT_V2 or LCR_DEPTH_PINHOLE_F32 (float32 mm) */
  int width, height;
  int frames;                /* burst length F >= 1; frames are fused by the zero-eliminated mean */
  double fx, fy, cx, cy;     /* intrinsics */
  double depth_min, depth_max; /* kept depth range in mm, inclusive */
  int roi_left, roi_right, roi_top, roi_bottom; /* kept pixel window, inclusive */
  double scale;              /* output units per mm (1: mm as the reference writes, 0.001: metres) */
  int normals;               /* pinhole models: 1 = image-gradient normals of depth_capture.cpp:231-265 */
  uint8_t r, g, b, pad;      /* constant colour (super_resolution.cpp:114 writes 128,128,128) */
} lcr_depth_params;

/* Burst fusion + back-projection: F frames of width*height depth (frame-major,
 * row-major) -> cloud of the kept pixels in row-major pixel order.
 * Replaces capture/super_resolution/super_resolution.cpp:295-309 (ZE mean) and
 * save_ply (:33-126), capture/depth_capture/depth_capture.cpp:216-317, and
 * capture/depth_capture_kv2/kinect2.h:144-201 + depth_capture_kv2.cpp:224-256
 * (V2: reprojection ROI + scale).  depth is a host pointer. */
LCR_API lcr_status lcr_backproject(lcr_ctx* ctx, const void* depth, const lcr_depth_params* p, lcr_cloud** out);
/* Same with the depth frames already on the context's device. */
LCR_API lcr_status lcr_backproject_device(lcr_ctx* ctx, const void* d_depth, const lcr_depth_params* p,
                                          lcr_cloud** out);
/* No counterpart in the reference.  lcr_backproject_device for callers that
 * cannot allocate device memory: a capture loop that runs in a fixed device-
 * memory budget next to the camera driver, or that must not stall in the
 * allocator between frames.  It allocates nothing: the kept pixels are written
 * as lcr_point records, in row-major pixel order, into d_points (caller-owned
 * device memory, capacity records), and their number to *d_count (a
 * caller-owned device uint32); records past capacity are not written, so
 * compare *d_count with capacity (capacity = width*height always suffices).
 * d_points must be 16-byte aligned and d_count 4-byte aligned (the records are
 * written as 16-byte vectors); other pointers return LCR_ERR_INVALID_ARG.
 * The points are the ones lcr_backproject_device gives, bit for bit.  The
 * scratch (the fused image of a burst and the compaction's block counts) is
 * one static device buffer of 1.2 MB per device, so width*height may be at
 * most 307200 (640x480); larger images return LCR_ERR_INVALID_ARG.  Nothing
 * in the scratch carries over between calls (every block count is written
 * before it is read), so it needs no clearing.  The first call on a device
 * looks up the scratch's address (cudaGetSymbolAddress): make it before any
 * stream capture.  The address is kept for the life of the process: after a
 * cudaDeviceReset (which unloads the module and its scratch) this entry point
 * must not be called again in that process.  All contexts on a device share
 * the scratch: calls that overlap in time (other streams, contexts or
 * threads) race on it.  Returns without synchronising; the results are ready
 * when the context's stream is. */
LCR_API lcr_status lcr_backproject_into(lcr_ctx* ctx, const void* d_depth, const lcr_depth_params* p,
                                        lcr_point* d_points, size_t capacity, uint32_t* d_count);
/* The fused (zero-eliminated mean) depth image alone, host in/out: uint16 for
 * V1 (super_resolution.cpp:295-315), float for V2 (super_resolution_kv2.cpp:287-303). */
LCR_API lcr_status lcr_burst_fuse(lcr_ctx* ctx, const void* frames, const lcr_depth_params* p, void* fused_out);

/* --------------------------------------------------------------- filters */
/* pcl::VoxelGrid<PointXYZRGBNormal> (pcl_tools/cloud_downsampling.cpp:73-76). */
LCR_API lcr_status lcr_voxel_grid(lcr_ctx* ctx, const lcr_cloud* in, float leaf_x, float leaf_y, float leaf_z,
                                  lcr_cloud** out);

typedef struct lcr_sor_stats {
  double mean, stddev, threshold;
  size_t valid, kept, removed;
} lcr_sor_stats;

/* pcl::StatisticalOutlierRemoval (pcl_tools/outlier_removal.cpp:80-84 and the
 * setNegative(true) pass :91-93).  inliers / outliers may each be NULL. */
LCR_API lcr_status lcr_sor(lcr_ctx* ctx, const lcr_cloud* in, int mean_k, double std_mul, lcr_cloud** inliers,
                           lcr_cloud** outliers, lcr_sor_stats* stats);
/* Per-point mean neighbour distance of the SOR first pass (host output, n floats). */
LCR_API lcr_status lcr_sor_distances(lcr_ctx* ctx, const lcr_cloud* in, int mean_k, float* distances,
                                     lcr_sor_stats* stats);

enum { LCR_NORMALS_FLIP_ALL = 1, LCR_NORMALS_KEEP_NEIGHBOURS = 2 };
/* pcl::NormalEstimation with k neighbours and a viewpoint
 * (pcl_tools/normal_estimation.cpp:84-118).  flags LCR_NORMALS_FLIP_ALL negates
 * every normal afterwards (the tool's centroid XOR reverse rule :112-118).
 * LCR_NORMALS_KEEP_NEIGHBOURS (k <= 31; ignored above) keeps every point's k
 * nearest neighbours with the output cloud (128 B per point, freed with it):
 * lcr_icp / lcr_icp_batch with that cloud as the target then settle most
 * correspondences from the previous iteration's one and its neighbour list
 * instead of a tree search, with the same result.
 * Output: the input cloud with normal_x/y/z and curvature replaced. */
LCR_API lcr_status lcr_normals(lcr_ctx* ctx, const lcr_cloud* in, int k, const float viewpoint[3], int flags,
                               lcr_cloud** out);

/* ------------------------------------------------------------------- ICP */
enum { LCR_ICP_POINT_TO_POINT = 0, LCR_ICP_POINT_TO_PLANE = 1 };

typedef struct lcr_icp_params {
  double max_correspondence_distance;   /* fine_registration.cpp:112 (default 0.1) */
  int max_iterations;                   /* :114 (default 50) */
  double transformation_epsilon;        /* :116 (default 1e-9) */
  double euclidean_fitness_epsilon;     /* :118 (default 0.001) */
  int method;                           /* LCR_ICP_POINT_TO_POINT (the tool's) or _TO_PLANE */
  int compute_fitness;                  /* 1: run getFitnessScore() after align (default) */
  /* No counterpart in PCL (0 = off, the default, PCL's behaviour): a pair whose
   * root-mean-square correspondence distance is still above stop_rms after
   * stop_iteration iterations ends there, not converged, with state
   * LCR_ICP_STATE_STOPPED -- a batch stops spending rounds on pairs that
   * cannot settle (views that share too little surface). */
  int stop_iteration;
  double stop_rms;
} lcr_icp_params;

enum {
  LCR_ICP_STATE_NOT_CONVERGED = 0,
  LCR_ICP_STATE_ITERATIONS = 1,
  LCR_ICP_STATE_TRANSFORM = 2,
  LCR_ICP_STATE_ABS_MSE = 3,
  LCR_ICP_STATE_REL_MSE = 4,
  LCR_ICP_STATE_NO_CORRESPONDENCES = 5,
  LCR_ICP_STATE_STOPPED = 6             /* the stop_iteration / stop_rms rule ended the pair */
};

typedef struct lcr_icp_result {
  float transform[16];       /* row-major final transformation (getFinalTransformation) */
  double transform64[16];    /* the same in FP64 */
  int converged;             /* hasConverged() */
  int iterations;
  int state;                 /* LCR_ICP_STATE_* */
  int n_correspondences;     /* of the last iteration */
  double fitness;            /* getFitnessScore() */
  double mse;                /* mean squared correspondence distance of the last iteration */
} lcr_icp_result;

LCR_API void lcr_icp_params_default(lcr_icp_params* p);
/* pcl::IterativeClosestPoint::align + getFinalTransformation + hasConverged +
 * getFitnessScore (pcl_tools/fine_registration.cpp:105-126).  guess may be
 * NULL (identity).  registered (may be NULL) receives the source transformed
 * by the final transformation, normals rotated (:121, :129). */
LCR_API lcr_status lcr_icp(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, const lcr_icp_params* p,
                           const float guess[16], lcr_icp_result* res, lcr_cloud** registered);

/* All pairs of a capture cycle at once (the reference runs fine_registration
 * once per pair, fine_registration.cpp:105-126): pair i aligns src[i] onto
 * tgt[i] with the shared parameters, from guesses + 16*i (row-major; guesses
 * may be NULL for identity).  The pairs iterate together over one work queue
 * (uneven sizes share the GPU) and each stops at its own convergence; each
 * result equals what lcr_icp gives for that pair alone.  Returns
 * LCR_ERR_NO_CORRESPONDENCES if some pair had too few (its result says so). */
LCR_API lcr_status lcr_icp_batch(lcr_ctx* ctx, const lcr_cloud* const* src, const lcr_cloud* const* tgt,
                                 size_t npairs, const lcr_icp_params* p, const float* guesses,
                                 lcr_icp_result* results);

/* One correspondence pass (for parity tests): source transformed by T
 * (row-major FP64, applied in FP32), exact nearest target within the maximum
 * distance; idx -1 when none.  Host outputs of length n_src. */
LCR_API lcr_status lcr_correspondences(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, const double T[16],
                                       double max_correspondence_distance, int32_t* idx, float* dist);

/* Exact k nearest neighbours of every query point in ref (squared FP32
 * distance as FLANN computes it, ties to the lower index).  max_dist_sq < 0:
 * uncapped.  Host outputs n_query*k, missing entries idx -1, dist +inf. */
LCR_API lcr_status lcr_knn(lcr_ctx* ctx, const lcr_cloud* ref, const lcr_cloud* query, int k, float max_dist_sq,
                           int32_t* idx, float* dist);

/* ------------------------------------------------------ SfM-side filters */
/* pcl::CropBox (pcl_tools/crop_cloud.cpp:81-97): inside = the finite points
 * with min <= p <= max on every axis, outside = the other finite points, each
 * in input order (either may be NULL). */
LCR_API lcr_status lcr_crop_box(lcr_ctx* ctx, const lcr_cloud* in, const float min[3], const float max[3],
                                lcr_cloud** inside, lcr_cloud** outside);
/* pcl::EuclideanClusterExtraction (pcl_tools/cluster_extraction.cpp:90-130):
 * connected components of the graph joining finite points whose squared FP32
 * distance is below float(tolerance^2) (FLANN's radius search), kept when
 * min_size <= size <= max_size, ordered by size (descending; equal sizes: the
 * cluster with the smaller first index first).  labels (host, n, may be NULL)
 * receives each point's cluster rank or -1; clustered the kept clusters'
 * points, cluster after cluster, ascending index within each; rest every
 * other point in input order (either may be NULL). */
LCR_API lcr_status lcr_euclidean_clusters(lcr_ctx* ctx, const lcr_cloud* in, double tolerance, size_t min_size,
                                          size_t max_size, int32_t* labels, size_t* nclusters, lcr_cloud** clustered,
                                          lcr_cloud** rest);
/* pcl::SACSegmentation with SACMODEL_PLANE, SAC_RANSAC and optimized
 * coefficients (pcl_tools/planar_segmentation.cpp:80-110): `hypotheses`
 * planes through three finite points drawn by a hash of seed, all scored at
 * once (inliers: |n.p + d| < threshold); the best (most inliers, then the
 * lowest hypothesis) is refitted by least squares on its inliers (FP64) and
 * the inliers are selected again.  coefficients (a b c d) of the refitted
 * plane; ninliers 0 when no plane was found.  plane: the inliers, rest: every
 * other point, in input order (either may be NULL). */
LCR_API lcr_status lcr_plane_segment(lcr_ctx* ctx, const lcr_cloud* in, double threshold, int hypotheses,
                                     uint64_t seed, float coefficients[4], size_t* ninliers, lcr_cloud** plane,
                                     lcr_cloud** rest);

/* ---------------------------------------------------- super-resolution */
/* The front end of capture/super_resolution/super_resolution.cpp:236-314 for
 * one view: frames (host, [frames][height][width] uint16 mm) are registered
 * to frame 0 by ECC affine alignment (enhanced correlation coefficient,
 * Gauss-Newton, after a 5x5 Gaussian smoothing, until the coefficient changes
 * by less than ecc_epsilon or after ecc_iterations), warped onto it
 * (bilinear, zero outside), upsampled by `factor` (nearest), fused by the
 * zero-eliminated mean and resampled back by Lanczos-4, rounded and
 * saturated to uint16 (depth_out [height][width]).  Optional outputs: warps
 * [frames][6] (2x3 row-major inverse maps, frame 0 the identity), minmax the
 * observed nonzero range, iterations [frames].  LCR_ERR_INVALID_ARG unless
 * 1 <= frames <= 1024, 1 <= factor <= 16, width * height <= 2^26,
 * ecc_iterations >= 0 and ecc_epsilon >= 0.  Synchronous: the outputs are
 * ready when the call returns. */
typedef struct lcr_sr_params {
  int width, height, frames;
  int factor;          /* resample factor (the tool's default 4) */
  int ecc_iterations;  /* 200 in the reference */
  double ecc_epsilon;  /* 1e-12 in the reference */
} lcr_sr_params;
LCR_API lcr_status lcr_super_resolve(lcr_ctx* ctx, const uint16_t* frames, const lcr_sr_params* p,
                                     uint16_t* depth_out, float* warps, float minmax[2], int32_t* iterations);
/* The Kinect v2 form (capture/super_resolution_kv2/super_resolution_kv2.cpp:
 * 222-311): float frames and a float fused image, not rounded; a pixel that no
 * frame covers is 0 (the reference leaves it uninitialised). */
LCR_API lcr_status lcr_super_resolve_f32(lcr_ctx* ctx, const float* frames, const lcr_sr_params* p,
                                         float* depth_out, float* warps, float minmax[2], int32_t* iterations);

/* ------------------------------------------------------------ autotuning */
/* Launch shapes of the search kernels.  Every result is independent of them;
 * only the speed changes. */
typedef struct lcr_tune {
  int sor_warps;          /* warps per block of the SOR k-NN kernel, 1-8 (default 5) */
  int normals_warps;      /* warps per block of the NormalEstimation k-NN kernels, 1-8 (default 5) */
  int icp_blocks_per_sm;  /* persistent blocks per SM of the batched ICP kernels, 1-8 (default 4) */
} lcr_tune;
LCR_API lcr_status lcr_tune_get(lcr_ctx* ctx, lcr_tune* t);
LCR_API lcr_status lcr_tune_set(lcr_ctx* ctx, const lcr_tune* t);

typedef struct lcr_tune_report {
  lcr_tune chosen;
  int from_cache;          /* 1: read from the cache file, nothing timed */
  double sor_ms[8];        /* SOR k-NN kernel time per candidate (index warps - 1; 0 = not a candidate) */
  double normals_ms[8];    /* NormalEstimation k-NN kernel time per candidate */
  double icp_ms[8];        /* one point-to-point ICP of src onto tgt per candidate blocks per SM */
} lcr_tune_report;
/* Times the candidate shapes on a representative pair (clouds of the size the
 * context will process: SOR k=50 and normals k=30 on src, ICP of src onto
 * tgt), applies the fastest, and when cache_path is not NULL appends the
 * choice there (one JSON object per line, keyed by the device name, its SM
 * count and floor(log2 n_src)); a later call with the same key reads the file
 * instead of timing.  src needs more than 50 points. */
LCR_API lcr_status lcr_autotune(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, const char* cache_path,
                                lcr_tune_report* report);

/* ------------------------------------------------ synthetic capture pairs */
/* Seeded capture pairs generated on the GPU (training and evaluation data of
 * the pose proposal): a superquadric object (semi-axes 0.05-0.2 m, exponents
 * 0.3-1.5) with a block and two balls attached, 1 m in front of the camera;
 * `points` visible surface samples per view (back-facing and covered points
 * dropped) with normals, depth noise sigma = 1.5 mm (z/1 m)^2 when noise is
 * set.  The target view moves the object about its centre by a yaw uniform
 * in +-yaw_deg, a tilt uniform in +-tilt_deg and a translation uniform in
 * +-translation (m) per axis; transforms [npairs][16] receives the exact
 * source-to-target transform (row-major).  npairs <= 65535. */
typedef struct lcr_synth_params {
  float yaw_deg, tilt_deg, translation;
  int noise;
} lcr_synth_params;
LCR_API lcr_status lcr_synthetic_pairs(lcr_ctx* ctx, uint64_t seed, size_t npairs, int points,
                                       const lcr_synth_params* p, lcr_cloud** src, lcr_cloud** tgt,
                                       float* transforms);

/* Depth images of the same objects (the seed and pair index pick the object,
 * its views and the exact transform as lcr_synthetic_pairs does).  Each
 * object's distance from the camera is distance[i] (m) when distance is given;
 * else, when points is given, the distance at which the object's mean
 * projected area (a quarter of its surface) covers points[i] pixels of this
 * camera, within [0.4, 8] m; with neither, 1 m.  Images:
 * the source and the target view of pair i are images 2i and 2i+1 of d_depth
 * (caller-owned device memory, [2 npairs][height][width]), uint16 mm for
 * LCR_DEPTH_KINECT_V1, float32 mm for LCR_DEPTH_KINECT_V2 and
 * LCR_DEPTH_PINHOLE_F32, 0 where no surface is seen.  The camera follows the
 * back-projection's conventions for the model (the reference's x = z(j-cx)/fx,
 * y = -z(i-cy)/fy looking down -z; Kinect v2 pixel centres at +0.5), so
 * lcr_backproject_device of an image gives points on the object's surface.
 * Surface samples are z-buffered, samples_per_pixel (0: 6) per frontal pixel
 * footprint; noise adds sigma = 1.5 mm (z/1 m)^2 per pixel.  transforms
 * [npairs][16] receives the exact source-to-target transforms.
 * Synchronises before returning.  npairs <= 32767. */
typedef struct lcr_render_params {
  int model;                 /* LCR_DEPTH_KINECT_V1, LCR_DEPTH_KINECT_V2 or LCR_DEPTH_PINHOLE_F32 */
  int width, height;
  double fx, fy, cx, cy;
  float samples_per_pixel;
} lcr_render_params;
LCR_API lcr_status lcr_synthetic_depth(lcr_ctx* ctx, uint64_t seed, size_t npairs, const lcr_synth_params* p,
                                       const lcr_render_params* camera, const float* distance,
                                       const float* points, void* d_depth, float* transforms);

/* A turntable cycle of one object (the object of pair 0 of lcr_synthetic_pairs
 * for this seed, its centre `distance` m in front of the camera): view v turns
 * it by v * step_deg about its vertical axis through its centre.  Images go to
 * d_depth [views][height][width] as for lcr_synthetic_depth; poses [views][16]
 * receives each view's object -> camera transform (row-major), so the
 * transform from view j into view i is poses[i] * inverse(poses[j]).  noise:
 * sigma = 1.5 mm (z/1 m)^2 per pixel.  Synchronises before returning.
 * views <= 65535. */
LCR_API lcr_status lcr_synthetic_turntable(lcr_ctx* ctx, uint64_t seed, int views, float step_deg,
                                           const lcr_render_params* camera, float distance, int noise,
                                           void* d_depth, float* poses);

/* Alignment error of n clouds: out[i] = RMS over the finite points p of
 * clouds[i] of |Ta_i p - Tb_i p| (FP64; Ta, Tb [n][16] row-major), the RMSE
 * by which a pair counts as aligned (estimate vs ground truth). */
LCR_API lcr_status lcr_rmse_batch(lcr_ctx* ctx, const lcr_cloud* const* clouds, size_t n, const double* Ta,
                                  const double* Tb, double* out);

/* ------------------------------------------------- learned pose proposal */
/* A shared-MLP point encoder (3 -> 64 -> 128 -> 1024 with ReLU, max over
 * LCR_POSENET_POINTS points sampled from each cloud, centred on its centroid
 * and scaled by 4/m) and a pair head (2048 -> 512 -> 256 -> 9: the first two
 * columns of R and a residual translation) propose the source-to-target
 * transform ICP starts from, in place of centroid_align's guess
 * (pcl_tools/centroid_align.cpp:102-130, alignment.sh:106-113).  bf16 weights
 * and activations with fp32 accumulation (the encoder on the tensor cores);
 * fp32 master weights, gradients and AdamW state, all on the GPU.  The
 * reference has no learned component: this is an addition beside the plain
 * path, which it leaves unchanged.  Parameters are one fp32 vector of
 * LCR_POSENET_PARAMS values: W1[64][3] b1 W2[128][64] b2 W3[1024][128] b3
 * H1[512][2048] c1 H2[256][512] c2 H3[9][256] c3 (row-major [out][in]). */
#define LCR_POSENET_PARAMS 1323401
#define LCR_POSENET_POINTS 1024
typedef struct lcr_posenet lcr_posenet;
typedef struct lcr_adamw_params {
  float lr, beta1, beta2, eps, weight_decay;
} lcr_adamw_params;

/* He-uniform initialisation from seed. */
LCR_API lcr_status lcr_posenet_create(lcr_ctx* ctx, uint64_t seed, lcr_posenet** net);
LCR_API lcr_status lcr_posenet_free(lcr_ctx* ctx, lcr_posenet* net);
/* Host copies of the fp32 parameter vector (LCR_POSENET_PARAMS floats). */
LCR_API lcr_status lcr_posenet_get_params(lcr_ctx* ctx, const lcr_posenet* net, float* params);
LCR_API lcr_status lcr_posenet_set_params(lcr_ctx* ctx, lcr_posenet* net, const float* params);
/* The network input of n clouds: pts [n][LCR_POSENET_POINTS][4] (x y z 0,
 * centred, scaled, bf16-valued) and centroids [n][3] (FP64), either may be NULL. */
LCR_API lcr_status lcr_posenet_sample(lcr_ctx* ctx, const lcr_cloud* const* clouds, size_t n, uint64_t seed,
                                      float* pts, double* centroids);
/* Forward pass on sampled input: pts [2*npairs][POINTS][4], the npairs source
 * clouds then the npairs target clouds.  Outputs (each may be NULL):
 * features [2*npairs][1024] pooled encoder outputs, argmax [2*npairs][1024]
 * winning point per channel (train = 1 only), out [npairs][9]. */
LCR_API lcr_status lcr_posenet_forward(lcr_ctx* ctx, lcr_posenet* net, const float* pts, size_t npairs, int train,
                                       float* features, int32_t* argmax, float* out);
/* Loss (mean over pairs of the squared error of the 9 outputs against labels
 * [npairs][9]) and its gradient (LCR_POSENET_PARAMS floats), no update. */
LCR_API lcr_status lcr_posenet_gradients(lcr_ctx* ctx, lcr_posenet* net, const float* pts, const float* labels,
                                         size_t npairs, float* loss, float* grads);
/* One AdamW step on a batch of pairs whose source-to-target transforms are
 * known (transforms [npairs][16], row-major). */
LCR_API lcr_status lcr_posenet_train_step(lcr_ctx* ctx, lcr_posenet* net, const lcr_cloud* const* src,
                                          const lcr_cloud* const* tgt, const float* transforms, size_t npairs,
                                          uint64_t seed, const lcr_adamw_params* opt, float* loss);
/* Proposed source-to-target transforms, guesses [npairs][16] row-major: the
 * input lcr_icp_batch takes. */
LCR_API lcr_status lcr_posenet_propose(lcr_ctx* ctx, lcr_posenet* net, const lcr_cloud* const* src,
                                       const lcr_cloud* const* tgt, size_t npairs, uint64_t seed, float* guesses);

/* ------------------------------------------------------------ accumulate */
enum { LCR_ACCUM_ALL = 1 };
/* accumulate_clouds (pcl_tools/accumulate_clouds.cpp:100-127): drop source
 * points inside the cube [q-r, q+r] of any target point q, clean the rest by
 * SOR(k, std_mul), output target followed by the remaining source.
 * LCR_ACCUM_ALL skips the crop and the SOR (:100).  remaining (may be NULL)
 * receives the remaining source (the --negative file, :130-134). */
LCR_API lcr_status lcr_accumulate(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, double radius, int k,
                                  double std_mul, int flags, lcr_cloud** out, lcr_cloud** remaining);
/* The crop predicate alone: removed[i] = 1 for redundant source points (host, n_src bytes). */
LCR_API lcr_status lcr_crop_redundant(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, double radius,
                                      uint8_t* removed);

/* ---------------------------------------------------- transforms, centroid */
/* pcl::removeNaNFromPointCloud (rotate_align/rotate_align.cpp:201): the points
 * with finite x, y, z, in their order. */
LCR_API lcr_status lcr_remove_nan(lcr_ctx* ctx, const lcr_cloud* in, lcr_cloud** out);
/* pcl::transformPointCloudWithNormals with a row-major 4x4 (pcl_tools/transform.cpp:90,
 * scale.cpp:70 with diag(s,s,s,1), and inside every ICP iteration). */
LCR_API lcr_status lcr_transform(lcr_ctx* ctx, const lcr_cloud* in, const float m[16], lcr_cloud** out);
/* pcl::compute3DCentroid (pcl_tools/centroid_align.cpp:105-109), FP64 accumulation. */
LCR_API lcr_status lcr_centroid(lcr_ctx* ctx, const lcr_cloud* in, float centroid[4]);
/* centroid_align (centroid_align.cpp:102-130): move the source centroid to the
 * origin, rotate by R_x(roll) R_y(pitch) R_z(yaw) (degrees), move to the target
 * centroid and add `elevation` along y.  Returns the transformed source and the
 * composed 4x4 (row-major). */
LCR_API lcr_status lcr_centroid_align(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, double roll,
                                      double pitch, double yaw, double elevation, lcr_cloud** out,
                                      float transform[16]);

/* ----------------------------------------------------------------- PLY I/O */
/* pcl::io::loadPLYFile<PointXYZRGBNormal> (e.g. pcl_tools/fine_registration.cpp:94):
 * ascii or binary PLY, any vertex layout; *pts is malloc'ed, release with
 * lcr_free.  Host only, no context or GPU needed. */
LCR_API lcr_status lcr_ply_read(const char* path, lcr_point** pts, size_t* n);
/* pcl::io::savePLYFileBinary (e.g. fine_registration.cpp:129): binary=1 writes
 * binary_little_endian, 0 ascii.  Fields x y z red green blue normal_x normal_y
 * normal_z curvature. */
LCR_API lcr_status lcr_ply_write(const char* path, const lcr_point* pts, size_t n, int binary);
/* Message of the last failing PLY call on this thread. */
LCR_API const char* lcr_ply_last_error(void);
LCR_API void lcr_free(void* p);

#ifdef __cplusplus
}
#endif
#endif /* LCR_H */
