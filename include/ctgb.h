/* ctgb.h — C ABI of the GB300 CT projection library (libctgb.so).
 *
 * Plain C: pointers, sizes, status codes.  Device pointers are CUDA global
 * memory owned by the caller; `stream` is a cudaStream_t passed as void*
 * (NULL = legacy default stream).  No entry point allocates device memory,
 * synchronises the device or exits the process.  Every entry point returns
 * CTGB_OK or a negative status; ctgb_last_error() gives the message of the
 * calling thread's last failure.  Projector calls take a view range
 * [view0, view0 + nviews) inside the scan; an empty range reads no
 * projections and writes none, so their pointers may then be NULL (a
 * backprojection without accumulate still clears the volume).
 *
 * Array layouts follow the reference (leehoy/CTReconstruction):
 *   volume      float32 [nz][ny][nx]      (Reconstruction.image)
 *   projections float32 [nviews][nv][nu]  (Reconstruction.proj)
 * y and z voxel indices run from +y/+z to -y/-z and detector rows from +z to
 * -z, as in python/Reconstruction_numba.py:813-815.
 */
#ifndef CTGB_H
#define CTGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CTGB_OK 0
#define CTGB_ERR_ARG (-1)      /* invalid argument / geometry                 */
#define CTGB_ERR_CUDA (-2)     /* CUDA launch or runtime error                */
#define CTGB_ERR_SIZE (-3)     /* buffer too small / size out of range        */
#define CTGB_ERR_TIMEOUT (-4)  /* a bounded device wait ran out               */

#define CTGB_FLAVOUR_NUMBA 0   /* python/Reconstruction_numba.py conventions  */
#define CTGB_FLAVOUR_PYCUDA 1  /* python/Reconstruction_pycuda.py conventions */

/* Scan geometry: the reference's params dict (Reconstruction_numba.py:58-62,
 * Reconstruction_pycuda.py:65-70), one field per key. */
typedef struct ctgb_params {
    int32_t nu, nv;                 /* NumberOfDetectorPixels                    */
    double du, dv;                  /* DetectorPixelSize                         */
    int32_t nx, ny, nz;             /* NumberOfImage                             */
    double dx, dy, dz;              /* ImagePixelSpacing                         */
    int32_t nviews;                 /* NumberOfViews                             */
    double start_angle, end_angle;  /* StartAngle, EndAngle (views: linspace(s,e,n+1)[:-1]) */
    double source_init[3];          /* SourceInit                                */
    double detector_init[3];        /* DetectorInit                              */
    double rotation_origin[3];      /* RotationOrigin                            */
    double phantom_center[3];       /* PhantomCenter                             */
    double recon_center[3];         /* ReconCenter                               */
    double detector_offset[2];      /* DetectorOffset (pycuda flavour only)      */
    double pitch;                   /* Pitch (helical)                           */
    int32_t curved;                 /* DetectorShape: 0 'Flat', 1 'Curved'       */
    int32_t flavour;                /* CTGB_FLAVOUR_*                            */
} ctgb_params;

/* ---- geometry tables -------------------------------------------------------
 * The per-view geometry the reference recomputes in NumPy on every call
 * (distance_forward Reconstruction_numba.py:834-908; distance_backproj
 * :405-413) is built once, in float64 on the host, into a flat table that the
 * caller copies to device memory and passes to the projectors. */
int ctgb_table_bytes(const ctgb_params *p, size_t *bytes);
/* On a full circular orbit whose view count is a multiple of 4, the view
 * records v + nviews/4 are stored as exact quarter-turn rotations of view v's
 * float values (rather than rounded independently, which differs by an ulp),
 * except in the groups of views containing a 45-degree tie of the forward's
 * dominant axis; the symmetric backprojectors rely on this. */
int ctgb_table_build(const ctgb_params *p, void *host_table, size_t bytes);

/* ---- DD forward projection -------------------------------------------------
 * Replaces Reconstruction.forward()/distance_forward (Reconstruction_numba.py
 * :793-1117) and the kernels distance_project_on_{x,y,z}
 * (GPUFuncs_numba.py:88-240; GPUFuncs_pycuda.py:398-588, *_3 variants).
 * proj[v-view0] = A vol for views [view0, view0+nviews).  vol_xzy is optional
 * (may be NULL): a copy of vol in [nz][nx][ny] order (ctgb_transpose_xy) that
 * lets x-dominant views read the volume with unit stride.  proj is
 * overwritten.  Stream-ordered; no synchronisation. */
int ctgb_forward(const ctgb_params *p, const void *d_table, const float *d_vol, const float *d_vol_xzy,
                 float *d_proj, int32_t view0, int32_t nviews, void *stream);
/* Number of kernel launches ctgb_forward makes for this view range: one for
 * all x-dominant and one for all y-dominant views (per 2048 views), and one
 * per run of consecutive z-dominant views. */
int ctgb_forward_launches(const ctgb_params *p, int32_t view0, int32_t nviews, int32_t *launches);
/* Detector rows per forward tile for this scan (host-only): 32 when a
 * detector row spans at most 1.3 voxel rows anywhere a ray meets the volume,
 * (dv / dz) * (SAD + |centre - origin| + in-plane half-diagonal) / SDD <= 1.3,
 * else 16.  Only speed depends on it; the projections do not. */
int ctgb_forward_tile_rows(const ctgb_params *p, int32_t *rows);

/* Same result as ctgb_forward, for callers that cannot allocate device
 * memory where they project (an application whose own pool owns the device
 * memory budget, or a latency-bound loop that cannot take cudaMalloc's
 * device-wide synchronisation).  No counterpart in the reference.  Instead of
 * a caller-allocated d_vol_xzy it uses a file-scope __device__ array of
 * CTGB_STATIC_MAX_VOXELS floats (16 MiB, held by every GPU that loads the
 * library until exit); larger volumes are rejected with CTGB_ERR_SIZE.  The
 * first call on a device looks up that array's address (make it before any
 * stream capture).  All calls share the array: calls that overlap on the GPU
 * race on it. */
#define CTGB_STATIC_MAX_VOXELS (1 << 22)
int ctgb_forward_static(const ctgb_params *p, const void *d_table, const float *d_vol, float *d_proj,
                        int32_t view0, int32_t nviews, void *stream);

/* vol_xzy[z][x][y] = vol[z][y][x]: the layout ctgb_forward reads for
 * x-dominant views.  No reference counterpart. */
int ctgb_transpose_xy(const float *d_vol, float *d_vol_xzy, int32_t nx, int32_t ny, int32_t nz, void *stream);

/* ---- FDK-weighted DD backprojection ---------------------------------------
 * Replaces Reconstruction.backward()/distance_backproj (Reconstruction_numba.py
 * :261-271, :371-482) and flat_/curved_distance_backproj_arb
 * (GPUFuncs_numba.py:391-686; GPUFuncs_pycuda.py:837-956 flat_..._arb2).
 * vol = (accumulate ? vol : 0) + scale * sum_v BP_v(proj[v-view0]) where the
 * reference's backward() uses scale = dtheta = angle[1]-angle[0].
 * No workspace: each voxel column walks up the detector rows under its
 * footprint once per view.  A call over every view of a full circular orbit
 * whose view count is a multiple of 4 (or 2), with a square (or even-height)
 * grid centred on the rotation axis and no helical pitch, computes each
 * (column, view) set-up once for the 4 (or 2) columns that a quarter (half)
 * turn maps onto each other. */
int ctgb_backproject_fdk(const ctgb_params *p, const void *d_table, const float *d_proj, float *d_vol,
                         int32_t view0, int32_t nviews, float scale, int32_t accumulate, void *stream);
/* ctgb_backproject_fdk over part of a symmetric orbit, for callers that feed
 * the views in pieces (e.g. while they arrive from host memory).
 * ctgb_backproject_fdk_orbit_size gives nc = 4, 2 or 1, the rotation-orbit
 * size that ctgb_backproject_fdk uses for a call over every view; the views
 * then split into base views b in [0, nviews/nc), and base view b stands for
 * the nc views b + k * nviews/nc.  ctgb_backproject_fdk_orbits backprojects
 * base views [base0, base0 + nbase): d_proj holds every view of the scan (at
 * least those nc slabs), indexed by absolute view.  Calls over base ranges
 * that tile [0, nviews/nc), the first with accumulate = 0 and the rest with
 * 1, give ctgb_backproject_fdk's result up to float summation order.
 * Replaces the same reference code as ctgb_backproject_fdk. */
int ctgb_backproject_fdk_orbit_size(const ctgb_params *p, int32_t *nc);
int ctgb_backproject_fdk_orbits(const ctgb_params *p, const void *d_table, const float *d_proj, float *d_vol,
                                int32_t base0, int32_t nbase, float scale, int32_t accumulate, void *stream);

/* Same result as ctgb_backproject_fdk: the projections are first integrated
 * along v into a caller-supplied workspace of float2 (running sum, value) per
 * detector cell and view, so each voxel's footprint costs two lookups per
 * detector column.  Views are processed in chunks that fit the workspace (at
 * least one view: ctgb_backproject_fdk_workspace_bytes(p, 1, ..)).  A call
 * that ctgb_backproject_fdk serves with four-fold symmetry goes there
 * instead (it is faster) and leaves the workspace untouched.
 * Replaces the same reference code as ctgb_backproject_fdk. */
/* Workspace bytes for nviews views of ctgb_backproject_fdk_ws and of
 * ctgb_backproject_matched_ws (the latter's per-view tables included). */
int ctgb_backproject_fdk_workspace_bytes(const ctgb_params *p, int32_t nviews, size_t *bytes);
int ctgb_backproject_fdk_ws(const ctgb_params *p, const void *d_table, const float *d_proj, float *d_vol,
                            int32_t view0, int32_t nviews, float scale, int32_t accumulate, void *d_workspace,
                            size_t workspace_bytes, void *stream);
/* The two stages of ctgb_backproject_fdk_ws as separate calls, so that one
 * set of integrated projections can serve several backprojections (and each
 * stage can be timed alone): ctgb_integrate_projections writes nviews views
 * of d_proj as (running sum, value) pairs into d_workspace (at least
 * ctgb_backproject_fdk_workspace_bytes(p, nviews) bytes);
 * ctgb_backproject_fdk_integrated backprojects nviews integrated views
 * (geometry of views view0 .. view0+nviews-1) from there. */
int ctgb_integrate_projections(const ctgb_params *p, const float *d_proj, int32_t nviews, void *d_workspace,
                               size_t workspace_bytes, void *stream);
int ctgb_backproject_fdk_integrated(const ctgb_params *p, const void *d_table, const void *d_integrated,
                                    float *d_vol, int32_t view0, int32_t nviews, float scale, int32_t accumulate,
                                    void *stream);

/* ---- matched DD backprojection (exact adjoint of ctgb_forward) -------------
 * No reference counterpart (the reference's backward() is FDK-weighted);
 * vol = (accumulate ? vol : 0) + scale * A^T proj. */
int ctgb_backproject_matched(const ctgb_params *p, const void *d_table, const float *d_proj, float *d_vol,
                             int32_t view0, int32_t nviews, float scale, int32_t accumulate, void *stream);
/* Same result, faster: projections prescaled by the forward's per-pixel
 * factor and integrated along v into a caller-supplied workspace, with a
 * per-view table of the forward's detector-column slopes and depth factors
 * after them (size per view from ctgb_backproject_fdk_workspace_bytes, which
 * counts both), processed in view chunks that fit.  A call over every view of
 * a quarter-turn-symmetric orbit (the conditions ctgb_backproject_fdk_orbit_size
 * reports as 4, plus forward planes centred on the axis) whose views all fit
 * takes one integration pass that stores the four views of each quarter-turn
 * orbit side by side per detector cell, one orbit-kernel launch, and one
 * launch per 45-degree group of views (whose dominant axes do not
 * alternate); the result is the chunked path's up to float summation order. */
int ctgb_backproject_matched_ws(const ctgb_params *p, const void *d_table, const float *d_proj, float *d_vol,
                                int32_t view0, int32_t nviews, float scale, int32_t accumulate, void *d_workspace,
                                size_t workspace_bytes, void *stream);

/* ---- FDK filtering ----------------------------------------------------------
 * Replaces Reconstruction.Filtering()/filter_proj/Filter
 * (Reconstruction_numba.py:190-259): cosine pre-weight, zero-padded ramp
 * filter along u, times deltaS.  filter_type: 0 ram-lak, 1 shepp-logan,
 * 2 cosine, 3 hamming, 4 hann.  ctgb_filter_bytes/ctgb_filter_build fill a
 * host buffer (the filter spectrum and cosine weights, float32) that the
 * caller copies to device memory once; ctgb_fdk_filter then filters
 * nrows_total = nviews*nv rows of proj in place. */
int ctgb_filter_bytes(const ctgb_params *p, size_t *bytes);
int ctgb_filter_build(const ctgb_params *p, int32_t filter_type, double cutoff, void *host_buf, size_t bytes);
int ctgb_fdk_filter(const ctgb_params *p, const void *d_filter, float *d_proj, int32_t nviews, void *stream);

/* ---- standalone cone-beam and fan-beam reconstructors ------------------------
 * Geometry of python/ConeBeam.py / ConeBeamGPU.py / FanBeam.py, read there from
 * a "key: value" text file (ReconstructionParams.txt, ConeBeam.py:57-84):
 * SourceToAxis, SourceToDetector, DetectorPixelWidth/Height,
 * DetectorWidth/Height (columns/rows), NumberOfViews, AngleCoverage (here in
 * radians), ReconVolume X*Y*Z.  For fan beam, DetectorHeight is the number of
 * slices and recon_z must equal it. */
typedef struct ctgb_conebeam_params {
    double source_to_axis, source_to_detector;
    double pixel_width, pixel_height;
    int32_t det_width, det_height;
    int32_t nviews;
    double angle_coverage;
    int32_t recon_x, recon_y, recon_z;
    int32_t arc;                    /* fan beam: 1 equiangular arc detector, 0 equispaced line */
} ctgb_conebeam_params;

/* Voxel-driven weighted FDK backprojection; replaces ConeBeamGPU.Reconstruction's
 * per-view CalculateInterpolGrid + Interpol2dLineargpu launches
 * (python/ConeBeamGPU.py:296-313; python/GPUFuncs_pycuda.py:40-102).
 * q: filtered projections [nviews][det_height][det_width]; recon: [Z][Y][X]. */
int ctgb_conebeam_table_bytes(const ctgb_conebeam_params *p, size_t *bytes);
int ctgb_conebeam_table_build(const ctgb_conebeam_params *p, void *host_table, size_t bytes);
int ctgb_conebeam_backproject(const ctgb_conebeam_params *p, const void *d_table, const float *d_q, float *d_recon,
                              int32_t view0, int32_t nviews, int32_t accumulate, void *stream);

/* Filter tables of the standalone reconstructors (ConeBeam.Filter / FanBeam.Filter,
 * python/ConeBeamGPU.py:353-379, python/FanBeam.py:175-209; arc kernel
 * matlab/FilterArc.m): variant 0 cone beam (cosine weight over u and v, rows
 * flipped along u as ConeBeamGPU.py:298 does), 1 fan line, 2 fan arc, 3 fan
 * arc with the balanced equiangular kernel (odd taps -1/(2 pi^2 sin^2(n tau)),
 * cutoff |w| > pi*cutoff; FilterArc.m's kernel keeps an extra tau^2 there).
 * Same layout as ctgb_filter_build; apply with ctgb_filter_apply. */
int ctgb_standalone_filter_bytes(const ctgb_conebeam_params *p, size_t *bytes);
int ctgb_standalone_filter_build(const ctgb_conebeam_params *p, int32_t variant, int32_t filter_type, double cutoff,
                                 void *host_buf, size_t bytes);
/* Filter nrows rows of length nu in place with a table from ctgb_filter_build
 * or ctgb_standalone_filter_build (rows grouped by nv rows per view for the
 * cosine weight).  zpl must equal ctgb_filter_zpl() of that table: it sizes
 * the launch's shared memory, and a kernel that finds another length in the
 * device table leaves the rows untouched and sets CTGB_DEVERR_ARG in the
 * device status word. */
int ctgb_filter_apply(const void *d_filter, int32_t zpl, float *d_rows, int64_t nrows, void *stream);
/* zpl (zero-padded row length) of a host filter table. */
int ctgb_filter_zpl(const void *host_buf, int32_t *zpl);

/* ---- batched 2-D fan-beam backprojection -------------------------------------
 * Many fan-beam slices of uneven image size in one persistent launch (the
 * per-slice backprojection of python/FanBeam.py:110-131, line detector, or
 * matlab/FanBeamReconArc.m:34-47, arc detector).  Each slice has its own
 * image grid, scan geometry and filtered sinogram [nviews][nch]; the work list
 * is (slice, tile) items of tile_x x tile_y pixels. */
typedef struct ctgb_fan_slice {
    int32_t nx, ny;            /* image columns / rows; the image is [ny][nx] */
    float x0, dx, y0, dy;      /* pixel centres x = x0 + i*dx, y = y0 + j*dy (mm) */
    float R, D;                /* source-to-axis; line: SourceToDetector - R (the U weight) */
    float g0, dg;              /* detector samples: line iso-scaled positions (mm), arc angles (rad) */
    int32_t nch, nviews;
    float theta0, dtheta;      /* view angles theta0 + v*dtheta; dtheta also scales the sum */
    int32_t arc, pad;
    int64_t sino_offset;       /* floats from the sinogram base */
    int64_t image_offset;      /* floats from the image base */
} ctgb_fan_slice;

int ctgb_fan_batch_bytes(const ctgb_fan_slice *slices, int32_t nslices, int32_t tile_x, int32_t tile_y, size_t *bytes);
int ctgb_fan_batch_build(const ctgb_fan_slice *slices, int32_t nslices, int32_t tile_x, int32_t tile_y,
                         void *host_buf, size_t bytes);
/* images[slice] (+)= backprojection; grid_blocks persistent CTAs of tile_x*tile_y
 * threads (the tile the batch was built with); max_views >= every slice's nviews. */
int ctgb_fan_backproject(const void *d_batch, int32_t max_views, const float *d_sino, float *d_images,
                         int32_t tile_x, int32_t tile_y, int32_t grid_blocks, int32_t accumulate, void *stream);

/* ---- iterative update passes ------------------------------------------------
 * Element-wise float32 passes over n elements of device arrays, one per
 * update line of the reference drivers (the A / A^T products come from
 * ctgb_forward / ctgb_backproject_*):
 *   ctgb_sart_residual  out = (ax - p0) / (a1 + eps)            python/SART.py:51
 *   ctgb_sart_update    x = x_prev - alpha * (bp / norm1 + eps) python/SART.py:55
 *   ctgb_em_ratio       p0[ax == 0] = 0 (in place); ax -> eps where 0; out = p0 / ax
 *                                                               python/EM.py:36-39
 *   ctgb_em_update      x = x_prev * (bp / norm)                python/EM.py:41-42
 *   ctgb_pocs_residual  out = (p0 - ax) / (a1 + eps), 0 where a1 == 0
 *                                                               python/ASD_POCS.py:174-175
 *   ctgb_pocs_update    x = max(0, x_prev + beta * bp / (norm1 + eps)), bp -> 0 where norm1 == 0
 *                                                               python/ASD_POCS.py:177-179
 *   ctgb_tv_step        y = x - step * g / ||g|| with g = tv_grad(x) on the
 *                       interior of the [n0][n1][n2] array (python/ASD_POCS.py:55-77,
 *                       :186-189); y's border is x's; x != y.
 *   ctgb_sqdist         out[0] = sum (a - b)^2 (b may be NULL: sum a^2), as double
 *                       (the norms of python/ASD_POCS.py:183,189).
 * The update passes accept x == x_prev (in place).  Reductions are
 * deterministic: `partials` holds ctgb_partials_count(n) doubles, one per
 * block, summed in a fixed order. */
int ctgb_partials_count(int64_t n, int32_t *count);
int ctgb_sart_residual(const float *ax, const float *p0, const float *a1, float eps, float *out, int64_t n,
                       void *stream);
int ctgb_sart_update(const float *x_prev, const float *bp, const float *norm1, float alpha, float eps, float *x,
                     int64_t n, void *stream);
int ctgb_em_ratio(float *p0, const float *ax, float eps, float *out, int64_t n, void *stream);
int ctgb_em_update(const float *x_prev, const float *bp, const float *norm, float *x, int64_t n, void *stream);
int ctgb_pocs_residual(const float *p0, const float *ax, const float *a1, float eps, float *out, int64_t n,
                       void *stream);
int ctgb_pocs_update(const float *x_prev, const float *bp, const float *norm1, float beta, float eps, float *x,
                     int64_t n, void *stream);
int ctgb_tv_step(const float *x, float *y, int32_t n0, int32_t n1, int32_t n2, float eps, float step,
                 double *partials, void *stream);
int ctgb_sqdist(const float *a, const float *b, int64_t n, double *partials, double *out, void *stream);

/* ---- ray-driven (Siddon) projection -----------------------------------------
 * The `Method: 'Ray'` projector (Reconstruction_numba.py:788-789 and
 * :266-268, stubs there; algorithm of matlab/RayDrivenProjection3DSiddon.m
 * :55-180): proj = line integrals of vol along the rays from the source to
 * every pixel centre (same geometry table as ctgb_forward);
 * ctgb_ray_backproject: vol = (accumulate ? vol : 0) + scale * transpose. */
int ctgb_ray_forward(const ctgb_params *p, const void *d_table, const float *d_vol, float *d_proj, int32_t view0,
                     int32_t nviews, void *stream);
int ctgb_ray_backproject(const ctgb_params *p, const void *d_table, const float *d_proj, float *d_vol, int32_t view0,
                         int32_t nviews, float scale, int32_t accumulate, void *stream);

/* ---- learned proximal step: 3-D U-Net blocks ---------------------------------
 * No reference counterpart (the network stands in for ASD-POCS's TV descent,
 * python/ASD_POCS.py:186-190).  Activations bf16 [N][D][H][W][C] (channels
 * innermost), conv weights bf16 [27 taps][Cout][Cin] with tap =
 * (dz+1)*9 + (dy+1)*3 + (dx+1), fp32 accumulation.
 *
 * ctgb_unet_conv3d: 3x3x3 convolution, zero padding, on the tcgen05 tensor
 * cores.  Input = channel concat of x0 (c0 channels) and, when c1 > 0, x1
 * (c1 channels), c0, c1 in {16, 32, 64}; w0 / w1 are the weight blocks of
 * the two segments ([27][cout][c0], [27][cout][c1]); cout in {16, 32, 48,
 * 64, 96}.  mode 0: out bf16 = relu(conv + bias); mode 1: out fp32 = conv
 * (bias unused).  W must be 16, 32, 64 or a multiple of 128, and H a
 * multiple of 128 / min(W, 128). */
int ctgb_unet_conv3d(const void *x0, int32_t c0, const void *x1, int32_t c1, const void *w0, const void *w1,
                     const float *bias, void *out, int32_t cout, int32_t n, int32_t d, int32_t h, int32_t w,
                     int32_t mode, void *stream);
/* x fp32 [n][vps] -> bf16 [n][vps][16] with channel 0 = x / scale[sample]. */
int ctgb_unet_input(const float *x, const float *scale, void *out, int32_t n, int64_t vps, void *stream);
/* The first layer in one pass on CUDA cores: out bf16 [n][d][h][w][16] =
 * relu(conv(a) + bias) with a = bf16(x / scale[sample]), x fp32 [n][d][h][w]
 * — ctgb_unet_input followed by ctgb_unet_conv3d (mode 0) on its 16-channel
 * output, whose channels 1-15 are zero.  w0: the conv's bf16 weight block
 * [27][16][cin]; only input channel 0 is read.  N * D at most 65535. */
int ctgb_unet_first(const float *x, const float *scale, const void *w0, int32_t cin, const float *bias, void *out,
                    int32_t n, int32_t d, int32_t h, int32_t w, void *stream);
/* 2x2x2 average pooling and nearest 2x upsampling (bf16, c a multiple of 8;
 * d, h, w are the fine dims for pooling and the output dims for upsampling). */
int ctgb_unet_pool2(const void *in, void *out, int32_t n, int32_t d, int32_t h, int32_t w, int32_t c, void *stream);
int ctgb_unet_up2(const void *in, void *out, int32_t n, int32_t d, int32_t h, int32_t w, int32_t c, void *stream);
/* Gradients through a ReLU whose output is act (bf16 [nvox][c]), reading
 * channels go .. go+c-1 of a gradient with gs channels per voxel:
 * relu_grad (same level), pool2_grad (gp at the coarse level / 8, plus an
 * optional skip gradient; d, h, w fine dims), up2_grad (sum of the 8 fine
 * children; d, h, w coarse dims).  Outputs bf16 [.][c]. */
int ctgb_unet_relu_grad(const float *g, int32_t gs, int32_t go, const void *act, void *out, int64_t nvox, int32_t c,
                        void *stream);
int ctgb_unet_pool2_grad(const float *gp, const float *gskip, int32_t gs, int32_t go, const void *act, void *out,
                         int32_t n, int32_t d, int32_t h, int32_t w, int32_t c, void *stream);
int ctgb_unet_up2_grad(const float *g, int32_t gs, int32_t go, const void *act, void *out, int32_t n, int32_t d,
                       int32_t h, int32_t w, int32_t c, void *stream);
/* 1x1x1 head with residual: y = x + scale[sample] * (sum_c wb[c] a[c] + wb[16]).
 * head_grad: ga = relu'(a) * gy * scale * wb[c] (bf16) and per-block partial
 * sums [blocks][17] of (gy * scale * a[c], gy * scale); blocks from
 * ctgb_unet_head_grad_blocks. */
int ctgb_unet_head(const void *a, const float *wb, const float *x, const float *scale, float *y, int32_t n,
                   int64_t vps, void *stream);
int ctgb_unet_head_grad_blocks(int64_t total, int32_t *blocks);
int ctgb_unet_head_grad(const float *gy, const void *a, const float *wb, const float *scale, void *ga,
                        float *partials, int32_t n, int64_t vps, void *stream);
/* Weight gradient of one input segment: partials[chunk][27][cout][cin] of
 * sum_v g[v][co] x[v + tap][ci] (chunks from ctgb_unet_wgrad_chunks; the
 * caller sums over chunks).  cin, cout multiples of 8, at most 96, and
 * cin * cout <= 6144. */
int ctgb_unet_wgrad_chunks(int32_t n, int32_t d, int32_t h, int32_t w, int32_t *chunks);
int ctgb_unet_wgrad(const void *x, int32_t cin, const void *g, int32_t cout, float *partials, int32_t n, int32_t d,
                    int32_t h, int32_t w, void *stream);
/* Per-block channel sums of a bf16 [nvox][c] gradient (c <= 64) ->
 * partials[blocks][c] (the bias gradient after a sum over blocks). */
int ctgb_unet_colsum(const void *g, int32_t c, int64_t nvox, float *partials, int32_t blocks, void *stream);

/* ---- batched solver launches ------------------------------------------------
 * The iterative drivers (SART.py, EM.py, ASD_POCS.py and OS-SART, restated in
 * ctreconstruction_gb300/iterative.py) run one projector after the other per
 * update; the reference runs one scan at a time with one launch per view
 * (Reconstruction_numba.py:457-468, :1108-1112).  These entry points run the
 * forward projections, or the backprojections, of many scans of uneven sizes
 * in one persistent launch (a fixed grid of CTAs walking a work list of
 * (scan, view, detector tile) or (scan, voxel-column block) items), and fuse
 * the drivers' element-wise lines into the projectors' stores: the forward
 * can store a residual instead of A x, the backprojectors an updated iterate
 * instead of B r.  No reference counterpart as entry points; the fused lines
 * are SART.py:51,55, EM.py:36-42 and ASD_POCS.py:174-179.
 *
 * A plan is built once on the host (plan_bytes, then plan) from job
 * descriptions holding device pointers; the caller copies the host plan to a
 * device buffer of the same size and passes both to the launch function, which
 * reads launch sizes from the host copy and the jobs from the device copy (no
 * allocation, no host-to-device copy at launch).  Device plans are 128-byte
 * aligned.  ctas_per_sm sets the
 * persistent grid: min(items, SMs * ctas_per_sm) CTAs. */
#define CTGB_FWD_STORE 0          /* A x                                              */
#define CTGB_FWD_SART_RESIDUAL 1  /* (A x - p0) / (a1 + eps)                 SART.py:51 */
#define CTGB_FWD_POCS_RESIDUAL 2  /* (p0 - A x) / (a1 + eps), 0 where a1 == 0         */
#define CTGB_FWD_EM_RATIO 3       /* p0 / A x; where A x == 0: p0 := 0 in place, 0    */
#define CTGB_BP_STORE 0           /* vol = (accumulate ? vol : 0) + B r               */
#define CTGB_BP_SART_UPDATE 1     /* x = x - coef * (B r / n1 + eps)      SART.py:55 */
#define CTGB_BP_EM_UPDATE 2       /* x = x * (B r / n1)                   EM.py:41-42 */
#define CTGB_BP_POCS_UPDATE 3     /* x = max(0, x + coef * (n1 == 0 ? 0 : B r) / (n1 + eps)) */

typedef struct {
    const ctgb_params *params; /* the scan (host)                                         */
    const void *table;         /* its device geometry table                               */
    const float *vol;          /* device volume [nz][ny][nx]                              */
    float *vol_xzy;            /* device [nz][nx][ny] scratch the launch fills (x-dominant views read it); NULL: read vol */
    float *out;                /* device output of views view0 .. view0 + nviews - 1      */
    int32_t view0, nviews;
    int32_t epilogue;          /* CTGB_FWD_*                                              */
    float eps;
    float *p0;                 /* measured projections of those views (residual epilogues) */
    const float *a1;           /* A 1 of those views (SART and POCS residuals)            */
} ctgb_fwd_job;

int ctgb_batch_forward_plan_bytes(const ctgb_fwd_job *jobs, int32_t njobs, size_t *bytes);
int ctgb_batch_forward_plan(const ctgb_fwd_job *jobs, int32_t njobs, void *host_plan, size_t bytes);
/* Transposes (one launch) and forward-projects (one launch per dominant axis
 * and tile height present) every job of the plan. */
int ctgb_batch_forward(const void *host_plan, const void *d_plan, int32_t ctas_per_sm, void *stream);

typedef struct {
    const ctgb_params *params; /* the scan (host)                                         */
    const void *table;         /* its device geometry table                               */
    const float *proj;         /* device projections of views view0 .. view0 + nviews - 1 */
    float *vol;                /* device output volume (CTGB_BP_STORE)                    */
    void *workspace;           /* device scratch: ctgb_backproject_fdk_workspace_bytes(nviews), all views at once */
    size_t workspace_bytes;
    int32_t view0, nviews;
    float scale;               /* matched: vol = scale * A^T proj; FDK: the dtheta factor */
    int32_t accumulate;        /* CTGB_BP_STORE only                                      */
    int32_t epilogue;          /* CTGB_BP_*                                               */
    float coef, eps;
    float *x;                  /* iterate updated in place (update epilogues)             */
    const float *n1;           /* backprojection normaliser (update epilogues)            */
} ctgb_bp_job;

/* matched != 0: the matched (adjoint) backprojector of ctgb_backproject_matched_ws;
 * 0: the FDK-weighted one of ctgb_backproject_fdk_ws (all jobs flat, or all curved). */
int ctgb_batch_backproject_plan_bytes(const ctgb_bp_job *jobs, int32_t njobs, size_t *bytes);
int ctgb_batch_backproject_plan(const ctgb_bp_job *jobs, int32_t njobs, int32_t matched, void *host_plan,
                                size_t bytes);
/* Integrates (one launch) and backprojects (one launch) every job of the plan. */
int ctgb_batch_backproject(const void *host_plan, const void *d_plan, int32_t ctas_per_sm, void *stream);

/* ---- status ----------------------------------------------------------------
 * ctgb_device_status: the device-side status word of the current device
 * (CTGB_DEVERR_* bits set by kernels whose bounded waits ran out or that
 * refused a malformed device-side table).  Reads it
 * with a synchronous copy (so it synchronises the device) and optionally
 * clears it.  No reference counterpart (the reference has no device-side
 * error reporting). */
#define CTGB_DEVERR_TIMEOUT 1
#define CTGB_DEVERR_ARG 2      /* a kernel refused a malformed device-side table */
int ctgb_device_status(int32_t *out, int32_t clear);
/* Self-test of the bounded device waits every TMA/mbarrier kernel uses: one
 * warp waits, with a limit of `polls` polls (1 .. 2^20), on an mbarrier that
 * nothing arrives at; the wait runs out, sets CTGB_DEVERR_TIMEOUT in the
 * device status word, and the kernel returns (the context stays usable).
 * Stream-ordered.  No reference counterpart. */
int ctgb_selftest_bounded_wait(int32_t polls, void *stream);
/* The calling thread's last error message; replaces the reference's
 * ErrorDescription printouts followed by sys.exit()
 * (Reconstruction_numba.py:36-52). */
const char *ctgb_last_error(void);
/* Library version string.  No reference counterpart. */
const char *ctgb_version(void);

#ifdef __cplusplus
}
#endif
#endif /* CTGB_H */
