/* ctoracle.c — FP64 CPU restatement of the reference's distance-driven (DD)
 * projection path.  TEST INFRASTRUCTURE: only tests/, the smoke check and the
 * CPU-baseline leg of bench.py load this library, always as the checker,
 * never as the thing measured for the GPU path.
 *
 * Conventions restated from the reference (paths relative to its root):
 *   geometry:   python/Reconstruction_numba.py:57-90 (SAD, SDD, helical shift H)
 *   detector:   FlatDetectorConstruction :145-172, CurvedDetectorConstruction
 *               :121-143; pycuda flavour adds DetectorOffset and writes the v
 *               axis with the opposite sign (python/Reconstruction_pycuda.py:115-168)
 *   forward:    distance_forward :805-1117 (boundary lines, dominant axis,
 *               slopes/intercepts, intersection length) and the kernels
 *               distance_project_on_{x,y,z} python/GPUFuncs_numba.py:88-240
 *               (same maths as GPUFuncs_pycuda.py:398-588)
 *   weights:    weight_calculator1/2 GPUFuncs_numba.py:16-47 (eps clamp 1e-5
 *               numba, 1e-6 pycuda forward, none in flat_distance_backproj_arb2)
 *   backward:   distance_backproj :371-482 with flat_/curved_distance_backproj_arb
 *               GPUFuncs_numba.py:391-686 (= GPUFuncs_pycuda.py:837-956)
 * Every coordinate, slope and weight is evaluated in double precision; the
 * reference rounds its host-side tables to float32, so the two agree to
 * float32 rounding, not bit for bit.
 *
 * The matched backprojector is the literal transpose of ct_forward (same loop,
 * scatter instead of gather), so <A x, y> = <x, A^T y> holds to rounding.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int nx, ny, nz, nu, nv, nviews;
    double dx, dy, dz;          /* ImagePixelSpacing, as given (positive)           */
    double du, dv;              /* DetectorPixelSize                                */
    double sad, sdd;            /* |SourceInit-RotationOrigin|, |SourceInit-DetectorInit| */
    double src[3], det[3];      /* SourceInit, DetectorInit                         */
    double center_fwd[3];       /* PhantomCenter (numba) / ReconCenter (pycuda)     */
    double center_bp[3];        /* ReconCenter                                      */
    double det_offset[2];       /* DetectorOffset (pycuda flavour; zero for numba)  */
    double helical;             /* H = Pitch * nv * dv * SAD / SDD                  */
    int curved;                 /* DetectorShape == 'Curved'                        */
    int pycuda;                 /* 1: pycuda flavour sign/offset conventions        */
    double eps_fwd, eps_bp;     /* weight clamps: |w| < eps -> 0 (0 disables)       */
} ct_geom;

/* weight_calculator1 (descending planes) / weight_calculator2 (ascending). */
static double overlap(int ind, int s, int e, double c1, double c2, double d, double p_lo, double p_hi,
                      double eps) {
    double w;
    double lo = c1 < c2 ? c1 : c2, hi = c1 < c2 ? c2 : c1, len = fabs(c1 - c2);
    if (s == e)
        w = 1.0;
    else if (d < 0) {           /* weight_calculator1: plane index grows as the coordinate falls */
        if (ind == s) w = (hi - p_hi) / len;
        else if (ind == e) w = (p_lo - lo) / len;
        else w = fabs(d) / len;
    } else {                    /* weight_calculator2 */
        if (ind == s) w = (p_hi - lo) / len;
        else if (ind == e) w = (hi - p_lo) / len;
        else w = fabs(d) / len;
    }
    if (fabs(w) < eps) w = 0.0;
    return w;
}

/* Source and detector-centre positions of view theta (distance_forward :872-874). */
static void view_positions(const ct_geom *g, double th, double S[3], double D[3]) {
    double zs = g->helical * th / (2.0 * M_PI);
    S[0] = -g->sad * sin(th); S[1] = g->sad * cos(th); S[2] = g->src[2] + zs;
    D[0] = (g->sdd - g->sad) * sin(th); D[1] = -(g->sdd - g->sad) * cos(th); D[2] = g->det[2] + zs;
}

/* World position of detector point with in-plane coordinates (u index value,
 * v index value): u_val/v_val are the already-scaled coordinates. */
static void det_point(const ct_geom *g, const double S[3], double th, double u, double v, double P[3]) {
    double eu[3] = {cos(th), sin(th), 0.0}, ew[3] = {sin(th), -cos(th), 0.0};
    double vz = g->pycuda ? v : -v;  /* numba: - V*ev ; pycuda: + V*ev with V already negated */
    for (int k = 0; k < 3; ++k) {
        if (g->curved)
            P[k] = S[k] + g->sdd * sin(u) * eu[k] + g->sdd * cos(u) * ew[k];
        else
            P[k] = S[k] + u * eu[k] + g->sdd * ew[k];
    }
    P[2] += vz;
}

static double u_center(const ct_geom *g, int c) {
    double d = g->curved ? g->du / g->sdd : g->du;
    return (c - (g->nu - 1) / 2.0) * d + (g->pycuda ? g->det_offset[0] : 0.0);
}
static double u_bound(const ct_geom *g, int c) {
    double d = g->curved ? g->du / g->sdd : g->du;
    return (c - (g->nu - 1) / 2.0) * d - d / 2.0 + (g->pycuda ? g->det_offset[0] : 0.0);
}
/* v coordinate as used in det_point (numba: +, subtracted later; pycuda: negated, added). */
static double v_center(const ct_geom *g, int r) {
    if (g->pycuda) return (r - (g->nv - 1) / 2.0) * -g->dv + g->det_offset[1];
    return (r - (g->nv - 1) / 2.0) * g->dv;
}
static double v_bound(const ct_geom *g, int r) {
    if (g->pycuda) return (r - (g->nv - 1) / 2.0) * -g->dv + g->dv / 2.0 + g->det_offset[1];
    return (r - (g->nv - 1) / 2.0) * g->dv - g->dv / 2.0;
}

/* Per-view forward setup shared by ct_forward and ct_backproject_matched. */
typedef struct {
    int axis;                   /* 0 x, 1 y, 2 z dominant            */
    int b1, b2;                 /* the two transverse axes            */
    double S[3];
} fwd_view;

static fwd_view fwd_setup(const ct_geom *g, double th) {
    fwd_view f;
    double D[3];
    view_positions(g, th, f.S, D);
    double ax = fabs(f.S[0] - D[0]), ay = fabs(f.S[1] - D[1]), az = fabs(f.S[2] - D[2]);
    if (ax >= ay && ax >= az) { f.axis = 0; f.b1 = 1; f.b2 = 2; }
    else if (ay >= ax && ay >= az) { f.axis = 1; f.b1 = 0; f.b2 = 2; }
    else { f.axis = 2; f.b1 = 0; f.b2 = 1; }
    return f;
}

/* Footprint of pixel (r,c) on every slice of the dominant axis; calls
 * visit(voxel_linear_index, weight) for each overlapped voxel. */
typedef void (*visit_fn)(void *ctx, long vox, double w);

static void pixel_footprint(const ct_geom *g, const fwd_view *f, double th, int r, int c,
                            const double *plane[3], const double d[3], const int n[3], int is0, int is1,
                            visit_fn visit, void *ctx) {
    const double *S = f->S;
    double PU1[3], PU2[3], PC[3], B1[3], B2[3];
    /* U lines: x/y of the column boundaries c and c+1, z of the pixel centre. */
    det_point(g, S, th, u_bound(g, c), v_center(g, r), PU1);
    det_point(g, S, th, u_bound(g, c + 1), v_center(g, r), PU2);
    /* V lines: x/y of the pixel centre, z of the row boundaries r+1 and r. */
    det_point(g, S, th, u_center(g, c), v_center(g, r), PC);
    det_point(g, S, th, u_center(g, c), v_bound(g, r + 1), B1);
    det_point(g, S, th, u_center(g, c), v_bound(g, r), B2);
    int a = f->axis, b1 = f->b1, b2 = f->b2;
    /* U lines give the b1 coordinate (x for y/z-dominant, y for x-dominant),
     * V lines the b2 coordinate; their start points follow distance_forward. */
    double P1[3], P2[3], Q1[3], Q2[3];
    memcpy(P1, PU1, sizeof P1); memcpy(P2, PU2, sizeof P2);
    memcpy(Q1, PC, sizeof Q1); memcpy(Q2, PC, sizeof Q2);
    /* z of the U points is the pixel-centre z; x,y of the V points the pixel centre. */
    P1[2] = PC[2]; P2[2] = PC[2];
    Q1[2] = B1[2]; Q2[2] = B2[2];
    if (a == 2) {
        /* z-dominant: U lines carry x, V lines carry y (distance_forward :1030-1039). */
    }
    double sU1 = (S[b1] - P1[b1]) / (S[a] - P1[a]), iU1 = -sU1 * S[a] + S[b1];
    double sU2 = (S[b1] - P2[b1]) / (S[a] - P2[a]), iU2 = -sU2 * S[a] + S[b1];
    double sV1 = (S[b2] - Q1[b2]) / (S[a] - Q1[a]), iV1 = -sV1 * S[a] + S[b2];
    double sV2 = (S[b2] - Q2[b2]) / (S[a] - Q2[a]), iV2 = -sV2 * S[a] + S[b2];
    double t1 = (S[b1] - PC[b1]) / (S[a] - PC[a]), t2 = (S[b2] - PC[b2]) / (S[a] - PC[a]);
    double L = fabs(d[a]) / (cos(atan(t1)) * cos(atan(t2)));
    double eps = g->eps_fwd;
    /* Slices [is0, is1) of the dominant axis (all of them for the forward). */
    for (int is = is0; is < is1; ++is) {
        double pc = plane[a][is] + d[a] / 2.0;
        double c11 = sU1 * pc + iU1, c12 = sU2 * pc + iU2;
        double c21 = sV1 * pc + iV1, c22 = sV2 * pc + iV2;
        int i11 = (int)floor((c11 - plane[b1][0]) / d[b1]), i12 = (int)floor((c12 - plane[b1][0]) / d[b1]);
        int i21 = (int)floor((c21 - plane[b2][0]) / d[b2]), i22 = (int)floor((c22 - plane[b2][0]) / d[b2]);
        int s1 = i11 < i12 ? i11 : i12, e1 = i11 < i12 ? i12 : i11;
        int s2 = i21 < i22 ? i21 : i22, e2 = i21 < i22 ? i22 : i21;
        for (int k = s1; k <= e1; ++k) {
            if (k < 0 || k > n[b1] - 1) continue;
            double w1 = overlap(k, s1, e1, c11, c12, d[b1], plane[b1][k], plane[b1][k + 1], eps);
            for (int l = s2; l <= e2; ++l) {
                if (l < 0 || l > n[b2] - 1) continue;
                double w2 = overlap(l, s2, e2, c21, c22, d[b2], plane[b2][l], plane[b2][l + 1], eps);
                int idx[3];
                idx[a] = is; idx[b1] = k; idx[b2] = l;
                long vox = ((long)idx[2] * g->ny + idx[1]) * g->nx + idx[0];
                visit(ctx, vox, w1 * w2 * L);
            }
        }
    }
}

static void make_planes(const ct_geom *g, double *xp, double *yp, double *zp, double d[3]) {
    /* distance_forward :834-840: y and z spacings negated (descending axes). */
    d[0] = g->dx; d[1] = -g->dy; d[2] = -g->dz;
    const double *C = g->center_fwd;
    for (int i = 0; i <= g->nx; ++i) xp[i] = C[0] + (i - (g->nx - 1) / 2.0) * d[0] - d[0] / 2.0;
    for (int i = 0; i <= g->ny; ++i) yp[i] = C[1] + (i - (g->ny - 1) / 2.0) * d[1] - d[1] / 2.0;
    for (int i = 0; i <= g->nz; ++i) zp[i] = C[2] + (i - (g->nz - 1) / 2.0) * d[2] - d[2] / 2.0;
}

typedef struct { const float *vol; double acc; } gather_ctx;
static void gather_visit(void *p, long vox, double w) {
    gather_ctx *c = (gather_ctx *)p;
    c->acc += (double)c->vol[vox] * w;
}
typedef struct { double *vol; double val; } scatter_ctx;
static void scatter_visit(void *p, long vox, double w) {
    scatter_ctx *c = (scatter_ctx *)p;
    c->vol[vox] += c->val * w;
}

/* proj[(view-view0)][nv][nu] = A vol, views [view0, view0+nview). */
void ct_forward(const ct_geom *g, const double *angles, int view0, int nview, const float *vol, double *proj,
                int nthreads) {
    double *xp = malloc(sizeof(double) * (g->nx + 1)), *yp = malloc(sizeof(double) * (g->ny + 1)),
           *zp = malloc(sizeof(double) * (g->nz + 1));
    double d[3];
    make_planes(g, xp, yp, zp, d);
    const double *plane[3] = {xp, yp, zp};
    const int n[3] = {g->nx, g->ny, g->nz};
    long npix = (long)g->nu * g->nv;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (long t = 0; t < (long)nview * npix; ++t) {
        int v = (int)(t / npix) + view0;
        int r = (int)((t % npix) / g->nu), c = (int)(t % g->nu);
        fwd_view f = fwd_setup(g, angles[v]);
        gather_ctx ctx = {vol, 0.0};
        pixel_footprint(g, &f, angles[v], r, c, plane, d, n, 0, n[f.axis], gather_visit, &ctx);
        proj[t] = ctx.acc;
    }
    free(xp); free(yp); free(zp);
}

/* vol += A^T proj over views [view0, view0+nview): the exact transpose of
 * ct_forward.  Within a view every pixel's footprint on slice `is` of the
 * dominant axis touches only voxels of that slice, so threads own disjoint
 * slice ranges and scatter without races. */
void ct_backproject_matched(const ct_geom *g, const double *angles, int view0, int nview, const float *proj,
                            double *vol, int nthreads) {
    double *xp = malloc(sizeof(double) * (g->nx + 1)), *yp = malloc(sizeof(double) * (g->ny + 1)),
           *zp = malloc(sizeof(double) * (g->nz + 1));
    double d[3];
    make_planes(g, xp, yp, zp, d);
    const double *plane[3] = {xp, yp, zp};
    const int n[3] = {g->nx, g->ny, g->nz};
    long npix = (long)g->nu * g->nv;
    for (int v = view0; v < view0 + nview; ++v) {
        fwd_view f = fwd_setup(g, angles[v]);
        const int ns = n[f.axis];
        /* A few slice ranges per thread: each range repeats the pixels'
         * per-view set-up, so more ranges cost more. */
        const int want = 4 * (nthreads > 0 ? nthreads : 1);
        const int nchunk = ns < want ? ns : want;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
        for (int k = 0; k < nchunk; ++k) {
            const int is0 = (int)((long)ns * k / nchunk), is1 = (int)((long)ns * (k + 1) / nchunk);
            for (long p = 0; p < npix; ++p) {
                scatter_ctx ctx = {vol, (double)proj[(long)(v - view0) * npix + p]};
                if (ctx.val == 0.0) continue;
                pixel_footprint(g, &f, angles[v], (int)(p / g->nu), (int)(p % g->nu), plane, d, n, is0, is1,
                                scatter_visit, &ctx);
            }
        }
    }
    free(xp); free(yp); free(zp);
}

/* vol = sum_views FDK-weighted DD backprojection of proj*dtheta
 * (distance_backproj :371-482 + flat/curved_distance_backproj_arb). */
void ct_backproject_fdk(const ct_geom *g, const double *angles, int view0, int nview, double dtheta,
                        const float *proj, double *vol, int nthreads) {
    const int nx = g->nx, ny = g->ny, nz = g->nz, nu = g->nu, nv = g->nv;
    double dx = g->dx, dy = -g->dy, dz = -g->dz;
    double du = g->curved ? g->du / g->sdd : g->du, dv = -g->dv;
    double *ki = malloc(sizeof(double) * (nu + 1)), *pp = malloc(sizeof(double) * (nv + 1));
    for (int i = 0; i <= nu; ++i) ki[i] = (i - (nu - 1) / 2.0) * du + (g->pycuda ? g->det_offset[0] : 0.0);
    for (int i = 0; i <= nv; ++i) pp[i] = (i - (nv - 1) / 2.0) * dv + (g->pycuda ? g->det_offset[1] : 0.0);
    const double *C = g->center_bp;
    const double R = g->sad, eps = g->eps_bp;
    long nvox = (long)nx * ny * nz;
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (long t = 0; t < nvox; ++t) {
        int iz = (int)(t / ((long)nx * ny)), iy = (int)((t / nx) % ny), ix = (int)(t % nx);
        double xx = C[0] + (ix - (nx - 1) / 2.0) * dx;
        double yy = C[1] + (iy - (ny - 1) / 2.0) * dy;
        double zz = C[2] + (iz - (nz - 1) / 2.0) * dz;
        double acc = 0.0;
        for (int v = view0; v < view0 + nview; ++v) {
            double th = angles[v], cs = cos(th), sn = sin(th);
            double zs = g->helical * th / (2.0 * M_PI);
            double Sx = g->src[0], Sy = g->src[1], Sz = g->src[2] + zs, Dy = g->det[1];
            double yc = yy * cs - xx * sn;
            double umin = INFINITY, umax = -INFINITY, vmin = INFINITY, vmax = -INFINITY;
            for (int q = 0; q < 8; ++q) {
                double cx = xx + ((q & 1) ? dx / 2.0 : -dx / 2.0);
                double cy = yy + ((q & 2) ? dy / 2.0 : -dy / 2.0);
                double cz = zz + ((q & 4) ? dz / 2.0 : -dz / 2.0);
                double xr = cx * cs + cy * sn, yr = cy * cs - cx * sn;
                double su = (Sx - xr) / (Sy - yr), sv = (Sz - cz) / (Sy - yr);
                if (su < umin) umin = su;
                if (su > umax) umax = su;
                if (sv < vmin) vmin = sv;
                if (sv > vmax) vmax = sv;
            }
            double cu1, cu2;
            if (g->curved) { cu1 = -atan(umin); cu2 = -atan(umax); }
            else { cu1 = umin * Dy + (Sx - umin * Sy); cu2 = umax * Dy + (Sx - umax * Sy); }
            double cv1 = vmin * Dy + (Sz - vmin * Sy), cv2 = vmax * Dy + (Sz - vmax * Sy);
            int iu1 = (int)floor((cu1 - ki[0]) / du), iu2 = (int)floor((cu2 - ki[0]) / du);
            int iv1 = (int)floor((cv1 - pp[0]) / dv), iv2 = (int)floor((cv2 - pp[0]) / dv);
            int su_ = iu1 < iu2 ? iu1 : iu2, eu_ = iu1 < iu2 ? iu2 : iu1;
            int sv_ = iv1 < iv2 ? iv1 : iv2, ev_ = iv1 < iv2 ? iv2 : iv1;
            double W = R * R / ((R - yc) * (R - yc));
            const float *Q = proj + (long)(v - view0) * nu * nv;
            for (int k = sv_; k <= ev_; ++k) {
                if (k < 0 || k > nv - 1) continue;
                double w1 = overlap(k, sv_, ev_, cv1, cv2, dv, pp[k], pp[k + 1], eps);
                for (int l = su_; l <= eu_; ++l) {
                    if (l < 0 || l > nu - 1) continue;
                    double w2 = overlap(l, su_, eu_, cu1, cu2, du, ki[l], ki[l + 1], eps);
                    acc += (double)Q[(long)k * nu + l] * dtheta * w1 * w2 * W;
                }
            }
        }
        vol[t] += acc;
    }
    free(ki); free(pp);
}

/* ---- ray-driven (Siddon) projection -----------------------------------------
 * matlab/RayDrivenProjection3DSiddon.m:55-180 restated on the Python class's
 * geometry (the `Method: 'Ray'` branch of distance_forward,
 * python/Reconstruction_numba.py:788-789, traces from the source to each
 * detector pixel centre through the same voxel planes): parametric plane
 * crossings alpha = (plane - S) / (P - S) per axis, the entry/exit
 * [alpha_min, alpha_max] clipped to [0, 1], the crossings inside merged and
 * de-duplicated within 1e-6 (uniquetol), each segment's length
 * |P - S| * (alpha_{i+1} - alpha_i) times the voxel holding its midpoint. */
static int cmp_double(const void *a, const void *b) {
    double x = *(const double *)a, y = *(const double *)b;
    return (x > y) - (x < y);
}

typedef void (*ray_visit_fn)(void *ctx, long vox, double len);

static void siddon_ray(const ct_geom *g, const double S[3], const double P[3], const double *const plane[3],
                       const double d[3], const int n[3], double *buf, ray_visit_fn visit, void *ctx) {
    const double tol_min = 1e-6;
    double amin = 0.0, amax = 1.0;
    for (int a = 0; a < 3; ++a) {
        double den = P[a] - S[a];
        if (fabs(den) < tol_min) {
            /* parallel to the planes of this axis: inside or not at all */
            double lo = plane[a][0] < plane[a][n[a]] ? plane[a][0] : plane[a][n[a]];
            double hi = plane[a][0] < plane[a][n[a]] ? plane[a][n[a]] : plane[a][0];
            if (S[a] < lo || S[a] > hi) return;
            continue;
        }
        double a0 = (plane[a][0] - S[a]) / den, a1 = (plane[a][n[a]] - S[a]) / den;
        double lo = a0 < a1 ? a0 : a1, hi = a0 < a1 ? a1 : a0;
        if (lo > amin) amin = lo;
        if (hi < amax) amax = hi;
    }
    if (amin > amax || fabs(amin - amax) < tol_min) return;
    int m = 0;
    buf[m++] = amin;
    for (int a = 0; a < 3; ++a) {
        double den = P[a] - S[a];
        if (fabs(den) < tol_min) continue;
        for (int i = 0; i <= n[a]; ++i) {
            double al = (plane[a][i] - S[a]) / den;
            if (al > amin && al < amax) buf[m++] = al;
        }
    }
    buf[m++] = amax;
    qsort(buf, (size_t)m, sizeof(double), cmp_double);
    int k = 1;
    for (int i = 1; i < m; ++i)
        if (buf[i] - buf[k - 1] > tol_min) buf[k++] = buf[i];
    double d12 = sqrt((S[0] - P[0]) * (S[0] - P[0]) + (S[1] - P[1]) * (S[1] - P[1]) + (S[2] - P[2]) * (S[2] - P[2]));
    for (int i = 0; i + 1 < k; ++i) {
        double am = 0.5 * (buf[i] + buf[i + 1]);
        int idx[3];
        int ok = 1;
        for (int a = 0; a < 3; ++a) {
            double f = (S[a] + am * (P[a] - S[a]) - plane[a][0]) / d[a];
            if (fabs(f) <= tol_min) f = 0.0;
            idx[a] = (int)floor(f);
            if (idx[a] < 0 || idx[a] >= n[a]) ok = 0;
        }
        if (!ok) continue;
        visit(ctx, ((long)idx[2] * g->ny + idx[1]) * g->nx + idx[0], d12 * (buf[i + 1] - buf[i]));
    }
}

static void ray_planes(const ct_geom *g, double **xp, double **yp, double **zp, double d[3]) {
    *xp = malloc(sizeof(double) * (g->nx + 1));
    *yp = malloc(sizeof(double) * (g->ny + 1));
    *zp = malloc(sizeof(double) * (g->nz + 1));
    make_planes(g, *xp, *yp, *zp, d);
}

/* proj[(view-view0)][nv][nu] = ray sums of vol. */
void ct_ray_forward(const ct_geom *g, const double *angles, int view0, int nview, const float *vol, double *proj,
                    int nthreads) {
    double *xp, *yp, *zp, d[3];
    ray_planes(g, &xp, &yp, &zp, d);
    const double *plane[3] = {xp, yp, zp};
    const int n[3] = {g->nx, g->ny, g->nz};
    const long npix = (long)g->nu * g->nv;
    const int cap = g->nx + g->ny + g->nz + 8;
#pragma omp parallel num_threads(nthreads)
    {
        double *buf = malloc(sizeof(double) * cap);
#pragma omp for schedule(dynamic, 64)
        for (long t = 0; t < (long)nview * npix; ++t) {
            int v = (int)(t / npix) + view0;
            int r = (int)((t % npix) / g->nu), c = (int)(t % g->nu);
            double S[3], D[3], P[3];
            view_positions(g, angles[v], S, D);
            det_point(g, S, angles[v], u_center(g, c), v_center(g, r), P);
            gather_ctx ctx = {vol, 0.0};
            siddon_ray(g, S, P, plane, d, n, buf, gather_visit, &ctx);
            proj[t] = ctx.acc;
        }
        free(buf);
    }
    free(xp); free(yp); free(zp);
}

/* vol += transpose of ct_ray_forward applied to proj (serial). */
void ct_ray_backproject(const ct_geom *g, const double *angles, int view0, int nview, const float *proj,
                        double *vol) {
    double *xp, *yp, *zp, d[3];
    ray_planes(g, &xp, &yp, &zp, d);
    const double *plane[3] = {xp, yp, zp};
    const int n[3] = {g->nx, g->ny, g->nz};
    const long npix = (long)g->nu * g->nv;
    double *buf = malloc(sizeof(double) * (g->nx + g->ny + g->nz + 8));
    for (int v = view0; v < view0 + nview; ++v) {
        double S[3], D[3], P[3];
        view_positions(g, angles[v], S, D);
        for (long p = 0; p < npix; ++p) {
            scatter_ctx ctx = {vol, (double)proj[(long)(v - view0) * npix + p]};
            if (ctx.val == 0.0) continue;
            det_point(g, S, angles[v], u_center(g, (int)(p % g->nu)), v_center(g, (int)(p / g->nu)), P);
            siddon_ray(g, S, P, plane, d, n, buf, scatter_visit, &ctx);
        }
    }
    free(buf);
    free(xp); free(yp); free(zp);
}
