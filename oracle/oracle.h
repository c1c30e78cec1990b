/*
 * CPU oracle for the alignment path -- TEST INFRASTRUCTURE ONLY.
 *
 * This library restates, on the CPU, the arithmetic of the reference tools
 * (Eberty/LowCost3DReconstruction pcl_tools/ and capture/) and of the PCL
 * algorithms they call.  It exists to check the CUDA library (liblcr) and to
 * time a CPU baseline.  Nothing in the shipped library links or calls it.
 *
 * Parity status: UNPINNED.  The reference ships no tests, golden vectors or
 * fixtures, and its arithmetic lives in PCL/FLANN/Eigen/OpenCV, none of which
 * exist in this build environment.  The restatement follows the reference call
 * sites (cited per function) and the documented semantics of the PCL classes;
 * it is anchored by known-answer tests and by independent cross-checks
 * (scipy cKDTree neighbour sets, numpy FP64 SVD/eigh).
 *
 * Build: g++ -O2 -fPIC -shared -ffp-contract=off -fopenmp (see build recipe in
 * lowcost3dreconstruction_gb300/build.py).  -ffp-contract=off is required: the
 * FP32 distance and transform expressions must round like the separate
 * multiply/add instructions FLANN and Eigen emit on x86 without FMA.
 */
#ifndef LCR_ORACLE_H
#define LCR_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Byte-compatible with pcl::PointXYZRGBNormal (48 bytes) and with lcr_point. */
typedef struct orc_point {
  float x, y, z, pad0;
  float normal_x, normal_y, normal_z, pad1;
  uint8_t b, g, r, a;
  float curvature;
  float pad2[2];
} orc_point;

typedef struct orc_bp_params {
  int width, height;
  double fx, fy, cx, cy;
  double depth_min, depth_max;        /* inclusive kept range, mm */
  int roi_left, roi_right, roi_top, roi_bottom; /* inclusive pixel ROI */
  double scale;                        /* output units per mm */
  int normals;                         /* 1: image-gradient normals (kv1) */
  uint8_t r, g, b, pad;                /* constant colour */
} orc_bp_params;

typedef struct orc_icp_params {
  double max_corr_dist;
  int max_iterations;
  double transformation_epsilon;
  double euclidean_fitness_epsilon;
  int point_to_plane;                  /* 0: point-to-point SVD, 1: point-to-plane LLS */
  int min_correspondences;             /* PCL default 3 */
} orc_icp_params;

typedef struct orc_icp_result {
  double transform[16];                /* row-major final transformation */
  int converged;
  int iterations;
  int state;                           /* 1 iterations, 2 transform, 3 abs mse, 4 rel mse, 5 no corr */
  int n_corr_last;
  double fitness;                      /* getFitnessScore(): mean NN squared distance, uncapped */
  double mse_last;
} orc_icp_result;

int orc_version(void);
void orc_set_threads(int n);

/* capture/super_resolution/super_resolution.cpp:295-309 (+ :315 convertTo) */
void orc_ze_mean_u16(const uint16_t* frames, int nframes, size_t npix, uint16_t* out);
/* capture/super_resolution_kv2/super_resolution_kv2.cpp:287-303 */
void orc_ze_mean_f32(const float* frames, int nframes, size_t npix, float* out);
/* capture/depth_capture/depth_capture.cpp:231-265 */
void orc_image_normals_u16(const uint16_t* depth, int w, int h, float* nrm_out);
/* capture/depth_capture/depth_capture.cpp:267-308; ascii_roundtrip=1 reproduces the %.6lf text detour */
size_t orc_backproject_v1(const uint16_t* depth, const orc_bp_params* p, int ascii_roundtrip, orc_point* out);
/* capture/depth_capture_kv2/kinect2.h:144-201,256-267 + depth_capture_kv2.cpp:224-256 */
size_t orc_backproject_v2(const float* depth_mm, const orc_bp_params* p, orc_point* out);

/* Exact kNN (FLANN L2_Simple FP32 distance, lowest-index tie rule).  max_dist_sq < 0: uncapped.
 * Missing neighbours are reported as idx -1, dist +inf. */
int orc_knn(const orc_point* ref, size_t m, const orc_point* q, size_t n, int k,
            float max_dist_sq, int32_t* idx, float* dist);

/* pcl::VoxelGrid (cloud_downsampling.cpp:73-76).  Returns the output count; *overflow set
 * when PCL would refuse (output = input copy). out must hold n points. */
size_t orc_voxel_grid(const orc_point* in, size_t n, float lx, float ly, float lz, orc_point* out,
                      int* overflow);
/* Voxel index per point (-1 if skipped); used to compare membership. */
void orc_voxel_keys(const orc_point* in, size_t n, float lx, float ly, float lz, int64_t* keys);

/* pcl::StatisticalOutlierRemoval (outlier_removal.cpp:80-84).  sqrt_double: 0 float sqrt,
 * 1 double sqrt; sum_mode: 0 blocked order shared with the GPU, 1 PCL sequential order.
 * stats = {mean, stddev, threshold, valid}. keep[i] = 1 for inliers (setNegative(false)). */
int orc_sor(const orc_point* in, size_t n, int mean_k, double std_mul, int sqrt_double,
            int sum_mode, float* distances, uint8_t* keep, double* stats);

/* pcl::NormalEstimation (normal_estimation.cpp:84-118), FP64 covariance and eigen-solve.
 * vp: viewpoint; flip_all: apply the tool's global sign flip afterwards. */
int orc_normals(const orc_point* in, size_t n, int k, const float* vp, int flip_all, orc_point* out);

/* pcl::IterativeClosestPoint (fine_registration.cpp:105-126). */
int orc_icp(const orc_point* src, size_t ns, const orc_point* tgt, size_t nt,
            const orc_icp_params* prm, const double* guess, orc_icp_result* res);
double orc_fitness(const orc_point* src, size_t ns, const orc_point* tgt, size_t nt, const double* T);
/* One correspondence pass: src transformed by T (FP32 cast), capped NN. */
int orc_correspondences(const orc_point* src, size_t ns, const orc_point* tgt, size_t nt,
                        const double* T, double max_corr_dist, int32_t* idx, float* dist);

/* CropBox-radius redundancy mask (accumulate_clouds.cpp:100-111): removed[i]=1 when some target
 * point q has float(q-r) <= p <= float(q+r) on all axes; with at least one target point, a
 * non-finite source point, or every source point when some target point is non-finite (CropBox
 * drops non-finite points, and no NaN comparison puts a point outside a NaN box). Returns the
 * removed count. */
size_t orc_crop_redundant(const orc_point* src, size_t ns, const orc_point* tgt, size_t nt,
                          double radius, uint8_t* removed);

/* transformPointCloudWithNormals (transform.cpp:90) with a row-major float 4x4. */
void orc_transform(const orc_point* in, size_t n, const float* m, orc_point* out);
/* compute3DCentroid (centroid_align.cpp:105-109), sequential FP32. */
void orc_centroid(const orc_point* in, size_t n, float* c);

/* FP64 helpers exposed for tests (independent of the GPU implementations). */
void orc_svd3(const double* a, double* u, double* s, double* v);
/* Super-resolution front end of one view (sr_oracle.cpp): F frames of w x h,
 * uint16 (f32 = 0) or float (f32 = 1); out the fused image of the same type,
 * warps [F][6], iterations [F]. */
void orc_super_resolve(const void* frames, int f32, int F, int w, int h, int factor, int iters, double eps,
                       void* out, float* warps, int* iterations);
void orc_eig3(const double* a, double* evals, double* evecs);

#ifdef __cplusplus
}
#endif
#endif
