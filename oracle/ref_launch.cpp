// Launchers for the reference's CUDA-C kernels (python/GPUFuncs_pycuda.py)
// compiled as host C++ under oracle/ref_shim.h.  Test infrastructure and the
// timed CPU baseline: nothing in the product links this.
//
// Every launch is emulated as a 1-D grid (gridDim.y = blockDim.y = 1), so a
// kernel's linear thread id `y*gridDim.x*blockDim.x + x` equals the id the
// launcher assigns.  OpenMP splits the ids so that all ids writing the same
// output element run in one OS thread:
//   * DD forward (distance_project_on_{x,y,z}3, GFp:398-588): id = slice*N+pix
//     accumulates into Dest[pix + view*N]; OS threads split pix, slices run in
//     order inside one OS thread.
//   * backprojectors and FDK interpolation (GFp:837-1193, :40-102): id = voxel
//     owns Dest[id]; OS threads split voxels.
#include "ref_shim.h"
#include <omp.h>

thread_local ref_dim3 threadIdx, blockIdx, blockDim, gridDim;

// Kernel prototypes (definitions come from the extracted kernel text).
void distance_project_on_y3(float*, float*, float*, float*, float*, float*, float*, float*, float*, float*,
                            float*, float*, float*, float*, float*);
void distance_project_on_x3(float*, float*, float*, float*, float*, float*, float*, float*, float*, float*,
                            float*, float*, float*, float*, float*);
void distance_project_on_z3(float*, float*, float*, float*, float*, float*, float*, float*, float*, float*,
                            float*, float*, float*, float*, float*);
void flat_distance_backproj_arb2(float*, float*, float*, float*, float*, float*, float*, float*);
void flat_distance_backproj_arb(float*, float*, float*, float*, float*, float*, float*, float*, float, float,
                                float, float, float, float, float, float, int);
void curved_distance_backproj_arb(float*, float*, float*, float*, float*, float*, float*, float*, float, float,
                                  float, float, float, float, float, float, int);
void CalculateInterpolGrid(float*, float*, float*, float*, float*, float*, float*);
void Interpol2dLineargpu(float*, float*, float*, float*, float*, float*, float*, float*);

static const unsigned kBlock = 256;

static inline void set_thread(long tid, long total) {
    blockDim.x = kBlock; blockDim.y = 1; blockDim.z = 1;
    gridDim.x = (unsigned)((total + kBlock - 1) / kBlock); gridDim.y = 1; gridDim.z = 1;
    blockIdx.x = (unsigned)(tid / kBlock); blockIdx.y = 0; blockIdx.z = 0;
    threadIdx.x = (unsigned)(tid % kBlock); threadIdx.y = 0; threadIdx.z = 0;
}

extern "C" {

int ref_max_threads(void) { return omp_get_max_threads(); }

// axis: 0 = x-dominant (on_x3), 1 = y-dominant (on_y3), 2 = z-dominant (on_z3).
// n_slices = number of slices along the dominant axis; param[6]*param[7] = nu*nv.
void ref_dd_forward3(int axis, float *Dest, float *Src, float *s1, float *s2, float *s3, float *s4, float *i1,
                     float *i2, float *i3, float *i4, float *Xplane, float *Yplane, float *Zplane, float *inter,
                     float *param, int n_slices, int nthreads) {
    const long N = (long)param[6] * (long)param[7];
    const long total = N * n_slices;
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (long pix = 0; pix < N; ++pix) {
        for (long s = 0; s < n_slices; ++s) {
            set_thread(s * N + pix, total);
            if (axis == 0)
                distance_project_on_x3(Dest, Src, s1, s2, s3, s4, i1, i2, i3, i4, Xplane, Yplane, Zplane, inter, param);
            else if (axis == 1)
                distance_project_on_y3(Dest, Src, s1, s2, s3, s4, i1, i2, i3, i4, Xplane, Yplane, Zplane, inter, param);
            else
                distance_project_on_z3(Dest, Src, s1, s2, s3, s4, i1, i2, i3, i4, Xplane, Yplane, Zplane, inter, param);
        }
    }
}

// flat_distance_backproj_arb2: geometry in the 20-float params array (GFp:837-956).
// voxel0/nvox select a contiguous range of linear voxel ids (a bounded sample).
void ref_backproj_arb2(float *Dest, float *Src, float *xp, float *yp, float *zp, float *up, float *vp,
                       float *params, long voxel0, long nvox, int nthreads) {
    const long total = (long)params[3] * (long)params[4] * (long)params[5];
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (long t = voxel0; t < voxel0 + nvox; ++t) {
        set_thread(t, total);
        flat_distance_backproj_arb2(Dest, Src, xp, yp, zp, up, vp, params);
    }
}

// Scalar-argument variants (GFp:958-1193); curved != 0 selects the arc detector.
void ref_backproj_arb(int curved, float *Dest, float *Src, float *xp, float *yp, float *zp, float *up, float *vp,
                      float *params, float sx, float sy, float sz, float dx, float dy, float dz, float a1, float a2,
                      int view, int nthreads) {
    const long total = (long)params[3] * (long)params[4] * (long)params[5];
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (long t = 0; t < total; ++t) {
        set_thread(t, total);
        if (curved)
            curved_distance_backproj_arb(Dest, Src, xp, yp, zp, up, vp, params, sx, sy, sz, dx, dy, dz, a1, a2, view);
        else
            flat_distance_backproj_arb(Dest, Src, xp, yp, zp, up, vp, params, sx, sy, sz, dx, dy, dz, a1, a2, view);
    }
}

// ConeBeamGPU voxel-driven FDK pair (GFp:89-102 then GFp:40-87), one view.
void ref_fdk_interp_view(float *Dest, float *Q, float *ki, float *p, float *IX, float *IY, float *IW, float *tt,
                         float *ss, float *zz, float *grid_params, float *interp_params, int nthreads) {
    const long total = (long)grid_params[1] * (long)grid_params[2] * (long)grid_params[3];
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (long t = 0; t < total; ++t) {
        set_thread(t, total);
        CalculateInterpolGrid(IX, IY, IW, tt, ss, zz, grid_params);
        Interpol2dLineargpu(Dest, Q, ki, p, IX, IY, IW, interp_params);
    }
}

}  // extern "C"
