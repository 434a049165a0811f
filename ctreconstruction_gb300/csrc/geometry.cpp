// Host side of libctgb: geometry tables and FDK filter tables, built in
// float64 from the reference's params dict and rounded to float32 once.
//
// Restates the reference's per-call host code:
//   Reconstruction.__init__            python/Reconstruction_numba.py:57-90
//   Flat/CurvedDetectorConstruction     :121-172 (pycuda flavour :115-168 adds
//                                       DetectorOffset and flips the v sign)
//   distance_forward planes + per view  :834-896 (Xplane/Yplane/Zplane, source,
//                                       detector centre, dominant axis)
//   distance_backproj planes            :405-413 (Xpixel.., ki, p)
//   Filter / filter_proj                :190-259
#include <cmath>
#include <cstring>
#include <vector>

#include "ctgb_internal.h"
#include "status.h"

namespace ctgb {

static bool valid(const ctgb_params *p) {
    if (!p) return set_error(CTGB_ERR_ARG, "params is NULL"), false;
    if (p->nu < 1 || p->nv < 1 || p->nx < 1 || p->ny < 1 || p->nz < 1 || p->nviews < 1)
        return set_error(CTGB_ERR_ARG, "sizes must be positive"), false;
    if (!(p->du > 0 && p->dv > 0 && p->dx > 0 && p->dy > 0 && p->dz > 0))
        return set_error(CTGB_ERR_ARG, "pixel and voxel spacings must be positive"), false;
    if (p->flavour != CTGB_FLAVOUR_NUMBA && p->flavour != CTGB_FLAVOUR_PYCUDA)
        return set_error(CTGB_ERR_ARG, "unknown flavour"), false;
    double sdd = std::sqrt(std::pow(p->source_init[0] - p->detector_init[0], 2) +
                           std::pow(p->source_init[1] - p->detector_init[1], 2) +
                           std::pow(p->source_init[2] - p->detector_init[2], 2));
    if (!(sdd > 0)) return set_error(CTGB_ERR_ARG, "source and detector coincide"), false;
    return true;
}

static size_t table_floats(const ctgb_params *p, TableHeader *h) {
    size_t hdr = (sizeof(TableHeader) + 127) / 128 * 32;   // header padded to 128 B
    size_t off = hdr;
    auto take = [&](int64_t n) { int64_t o = off; off += (n + 31) / 32 * 32; return o; };
    h->off_xplane = take(p->nx + 1);
    h->off_yplane = take(p->ny + 1);
    h->off_zplane = take(p->nz + 1);
    h->off_xpix = take(p->nx);
    h->off_ypix = take(p->ny);
    h->off_zpix = take(p->nz);
    h->off_ki = take(p->nu + 1);
    h->off_pp = take(p->nv + 1);
    ViewOffsets vo = view_offsets(p->nu, p->nv);
    h->view_stride = vo.stride;
    h->off_views = off;
    off += (size_t)vo.stride * p->nviews;
    return off;
}

struct Scan {
    double sad, sdd, H;
    std::vector<double> angles;
};

static Scan scan_of(const ctgb_params *p) {
    Scan s;
    const double *S = p->source_init, *D = p->detector_init, *O = p->rotation_origin;
    s.sad = std::sqrt((S[0] - O[0]) * (S[0] - O[0]) + (S[1] - O[1]) * (S[1] - O[1]) + (S[2] - O[2]) * (S[2] - O[2]));
    s.sdd = std::sqrt((S[0] - D[0]) * (S[0] - D[0]) + (S[1] - D[1]) * (S[1] - D[1]) + (S[2] - D[2]) * (S[2] - D[2]));
    s.H = p->pitch * (p->nv * p->dv) * s.sad / s.sdd;
    // numpy.linspace(start, end, n+1)[:-1]: start + i * ((end-start)/n)
    double step = (p->end_angle - p->start_angle) / p->nviews;
    s.angles.resize(p->nviews);
    for (int i = 0; i < p->nviews; ++i) s.angles[i] = i * step + p->start_angle;
    return s;
}

// Dominant axis of the forward projector at view angle th
// (distance_forward, python/Reconstruction_numba.py:896, :966).
static int view_axis(const ctgb_params *p, const Scan &s, double th) {
    const double zs = s.H * th / (2 * M_PI);
    const double S[3] = {-s.sad * std::sin(th), s.sad * std::cos(th), p->source_init[2] + zs};
    const double D[3] = {(s.sdd - s.sad) * std::sin(th), -(s.sdd - s.sad) * std::cos(th), p->detector_init[2] + zs};
    const double ax = std::fabs(S[0] - D[0]), ay = std::fabs(S[1] - D[1]), az = std::fabs(S[2] - D[2]);
    return (ax >= ay && ax >= az) ? 0 : (ay >= ax && ay >= az) ? 1 : 2;
}

bool quarter_turn_views(const ctgb_params *p, std::vector<int> *broken) {
    const int n = p->nviews, q = n / 4;
    if (broken) broken->clear();
    if (n < 4 || n % 4 || p->pitch != 0.0) return false;
    const Scan s = scan_of(p);
    std::vector<char> bad(q, 0);
    for (int v = 0; v < n; ++v) {
        const int w = (v + q) % n;
        const double a = s.angles[v], b = s.angles[w];
        const float ca = (float)std::cos(a), sa = (float)std::sin(a), cb = (float)std::cos(b), sb = (float)std::sin(b);
        if (std::fabs(cb + sa) > 2.4e-7f || std::fabs(sb - ca) > 2.4e-7f) return false;
        const int xa = view_axis(p, s, a), xb = view_axis(p, s, b);
        if (xa == 2 || xb != 1 - xa) bad[v % q] = 1;
    }
    if (broken)
        for (int g = 0; g < q; ++g)
            if (bad[g]) broken->push_back(g);
    return true;
}

bool slice_centres_antisymmetric(const ctgb_params *p) {
    if (p->nx != p->ny || p->dx != p->dy) return false;
    const bool pyc = p->flavour == CTGB_FLAVOUR_PYCUDA;
    const double *C = pyc ? p->recon_center : p->phantom_center;
    const int n = p->nx;
    const double dx = p->dx, dy = -p->dy;
    const float fdx = (float)dx, fdy = (float)dy;
    // the forward's slice centres as the kernels form them: plane + 0.5f * spacing
    auto fx = [&](int i) { return (float)(C[0] + (i - (n - 1) / 2.0) * dx - dx / 2) + 0.5f * fdx; };
    auto fy = [&](int i) { return (float)(C[1] + (i - (n - 1) / 2.0) * dy - dy / 2) + 0.5f * fdy; };
    for (int i = 0; i < n; ++i) {
        const float a = fx(i);
        if (fy(n - 1 - i) != a || fx(n - 1 - i) != -a || fy(i) != -a) return false;
    }
    return true;
}

}  // namespace ctgb

using namespace ctgb;

extern "C" int ctgb_table_bytes(const ctgb_params *p, size_t *bytes) {
    clear_error();
    if (!valid(p)) return last_status();
    if (!bytes) return set_error(CTGB_ERR_ARG, "bytes is NULL");
    TableHeader h;
    *bytes = table_floats(p, &h) * sizeof(float);
    return CTGB_OK;
}

extern "C" int ctgb_table_build(const ctgb_params *p, void *host_table, size_t bytes) {
    clear_error();
    if (!valid(p)) return last_status();
    TableHeader h;
    std::memset(&h, 0, sizeof h);
    size_t need = table_floats(p, &h) * sizeof(float);
    if (!host_table || bytes < need) return set_error(CTGB_ERR_SIZE, "table buffer too small");
    std::memset(host_table, 0, need);
    float *T = static_cast<float *>(host_table);
    const bool pyc = p->flavour == CTGB_FLAVOUR_PYCUDA;
    Scan s = scan_of(p);
    const int nx = p->nx, ny = p->ny, nz = p->nz, nu = p->nu, nv = p->nv;

    h.nx = nx; h.ny = ny; h.nz = nz; h.nu = nu; h.nv = nv; h.nviews = p->nviews;
    h.curved = p->curved ? 1 : 0;
    h.flavour = p->flavour;
    // weight_calculator1/2 clamp 1e-5 (GPUFuncs_numba.py:19,36); pycuda forward
    // 1e-6 (GPUFuncs_pycuda.py:436), flat_distance_backproj_arb2 none.
    h.eps_fwd = pyc ? 1e-6f : 1e-5f;
    h.eps_bp = pyc ? 0.0f : 1e-5f;
    const double dx = p->dx, dy = -p->dy, dz = -p->dz;   // Reconstruction_numba.py:813-815
    h.dx = (float)dx; h.dy = (float)dy; h.dz = (float)dz;
    const double du_bp = p->curved ? p->du / s.sdd : p->du, dv_bp = -p->dv;
    h.du_bp = (float)du_bp; h.dv_bp = (float)dv_bp;
    h.sad = (float)s.sad; h.sdd = (float)s.sdd;
    h.src0x = (float)p->source_init[0]; h.src0y = (float)p->source_init[1]; h.src0z = (float)p->source_init[2];
    h.det0y = (float)p->detector_init[1];
    h.dtheta = p->nviews > 1 ? (float)(s.angles[1] - s.angles[0]) : 0.0f;
    const double du_f = p->curved ? p->du / s.sdd : p->du;
    const double uoff = pyc ? p->detector_offset[0] : 0.0, voff = pyc ? p->detector_offset[1] : 0.0;
    h.du_fwd = (float)du_f;
    h.dv_fwd = (float)p->dv;
    h.u0_fwd = (float)((0 - (nu - 1) / 2.0) * du_f - du_f / 2.0 + uoff);

    // Forward planes: distance_forward :834-840 (pycuda :792-797 uses ReconCenter).
    const double *C = pyc ? p->recon_center : p->phantom_center;
    for (int i = 0; i <= nx; ++i) T[h.off_xplane + i] = (float)(C[0] + (i - (nx - 1) / 2.0) * dx - dx / 2);
    for (int i = 0; i <= ny; ++i) T[h.off_yplane + i] = (float)(C[1] + (i - (ny - 1) / 2.0) * dy - dy / 2);
    for (int i = 0; i <= nz; ++i) T[h.off_zplane + i] = (float)(C[2] + (i - (nz - 1) / 2.0) * dz - dz / 2);
    // Backprojector voxel centres and detector planes: distance_backproj :409-413.
    const double *RC = p->recon_center;
    for (int i = 0; i < nx; ++i) T[h.off_xpix + i] = (float)(RC[0] + (i - (nx - 1) / 2.0) * dx);
    for (int i = 0; i < ny; ++i) T[h.off_ypix + i] = (float)(RC[1] + (i - (ny - 1) / 2.0) * dy);
    for (int i = 0; i < nz; ++i) T[h.off_zpix + i] = (float)(RC[2] + (i - (nz - 1) / 2.0) * dz);
    for (int i = 0; i <= nu; ++i) T[h.off_ki + i] = (float)((i - (nu - 1) / 2.0) * du_bp + uoff);
    for (int i = 0; i <= nv; ++i) T[h.off_pp + i] = (float)((i - (nv - 1) / 2.0) * dv_bp + voff);

    ViewOffsets vo = view_offsets(nu, nv);
    for (int v = 0; v < p->nviews; ++v) {
        float *V = T + h.off_views + (int64_t)v * h.view_stride;
        const double th = s.angles[v];
        const double zs = s.H * th / (2 * M_PI);
        const double S[3] = {-s.sad * std::sin(th), s.sad * std::cos(th), p->source_init[2] + zs};
        const double D[3] = {(s.sdd - s.sad) * std::sin(th), -(s.sdd - s.sad) * std::cos(th),
                             p->detector_init[2] + zs};
        const double ax = std::fabs(S[0] - D[0]), ay = std::fabs(S[1] - D[1]), az = std::fabs(S[2] - D[2]);
        int axis = (ax >= ay && ax >= az) ? 0 : (ay >= ax && ay >= az) ? 1 : 2;   // :896, :966
        const double eu[2] = {std::cos(th), std::sin(th)}, ew[2] = {std::sin(th), -std::cos(th)};
        V[VF_AXIS] = (float)axis;
        V[VF_SX] = (float)S[0]; V[VF_SY] = (float)S[1]; V[VF_SZ] = (float)S[2];
        V[VF_COS] = (float)std::cos(th); V[VF_SIN] = (float)std::sin(th);
        V[VF_BPSZ] = (float)(p->source_init[2] + zs);
        V[VF_ANGLE] = (float)th;
        V[VF_EUX] = (float)eu[0]; V[VF_EUY] = (float)eu[1];
        V[VF_EWX] = (float)ew[0]; V[VF_EWY] = (float)ew[1];
        // Detector points (stored as float32 like the reference's DetectorIndex /
        // DetectorBoundary arrays).
        auto xy_of = [&](double u, double *x, double *y) {
            if (p->curved) {
                *x = S[0] + s.sdd * std::sin(u) * eu[0] + s.sdd * std::cos(u) * ew[0];
                *y = S[1] + s.sdd * std::sin(u) * eu[1] + s.sdd * std::cos(u) * ew[1];
            } else {
                *x = S[0] + u * eu[0] + s.sdd * ew[0];
                *y = S[1] + u * eu[1] + s.sdd * ew[1];
            }
        };
        for (int c = 0; c <= nu; ++c) {
            double x, y, u = (c - (nu - 1) / 2.0) * du_f - du_f / 2.0 + uoff;
            xy_of(u, &x, &y);
            V[vo.bx + c] = (float)x; V[vo.by + c] = (float)y;
        }
        for (int c = 0; c < nu; ++c) {
            double x, y, u = (c - (nu - 1) / 2.0) * du_f + uoff;
            xy_of(u, &x, &y);
            V[vo.px + c] = (float)x; V[vo.py + c] = (float)y;
        }
        // numba: z = S_z - v with v = (r-(nv-1)/2)*dv (-+ dv/2 for boundaries);
        // pycuda: z = S_z + v with v = (r-(nv-1)/2)*(-dv) (+ dv/2) + offset.
        auto zb = [&](int r) {
            return pyc ? S[2] + ((r - (nv - 1) / 2.0) * -p->dv + p->dv / 2.0 + voff)
                       : S[2] - ((r - (nv - 1) / 2.0) * p->dv - p->dv / 2.0);
        };
        for (int r = 0; r <= nv; ++r) V[vo.bz + r] = (float)zb(r);
        // Row-boundary model in the forward's z units (dz is the signed spacing).
        {
            const double b0 = (S[2] - zb(0)) / dz, bn = (S[2] - zb(nv)) / dz;
            V[VF_B0] = (float)b0;
            V[VF_DB] = (float)((bn - b0) / nv);
        }
        for (int r = 0; r < nv; ++r) {
            double z = pyc ? S[2] + ((r - (nv - 1) / 2.0) * -p->dv + voff) : S[2] - (r - (nv - 1) / 2.0) * p->dv;
            V[vo.pz + r] = (float)z;
        }
    }
    // A full circular orbit with a view count divisible by 4: rebuild views
    // v + Q (Q = views / 4) as exact quarter-turn rotations, (x, y) -> (-y, x),
    // of view v's float values, except in groups {g + k Q} where the forward's
    // dominant axis does not alternate (45-degree views, where the reference's
    // tie-break slices two views of the group along x).  Independently rounded, the two records differ
    // by an ulp (6e-5 mm at a 1000 mm source distance, 1e-4 of a detector
    // pixel); rotated exactly, every float expression of the forward projector
    // gives view v + Q the numbers it gives view v, so the matched
    // backprojector may share set-ups between the columns of a rotation orbit
    // and still be the forward's exact transpose.
    std::vector<int> broken;
    if (quarter_turn_views(p, &broken)) {
        const int q = p->nviews / 4;
        std::vector<char> bad(q, 0);
        for (int g : broken) bad[g] = 1;
        for (int v = q; v < p->nviews; ++v) {
            if (bad[v % q]) continue;   // a 45-degree tie: the reference slices both views along x
            const float *A = T + h.off_views + (int64_t)(v - q) * h.view_stride;
            float *V = T + h.off_views + (int64_t)v * h.view_stride;
            V[VF_SX] = -A[VF_SY]; V[VF_SY] = A[VF_SX];
            V[VF_COS] = -A[VF_SIN]; V[VF_SIN] = A[VF_COS];
            V[VF_EUX] = -A[VF_EUY]; V[VF_EUY] = A[VF_EUX];
            V[VF_EWX] = -A[VF_EWY]; V[VF_EWY] = A[VF_EWX];
            for (int c = 0; c <= nu; ++c) { V[vo.bx + c] = -A[vo.by + c]; V[vo.by + c] = A[vo.bx + c]; }
            for (int c = 0; c < nu; ++c) { V[vo.px + c] = -A[vo.py + c]; V[vo.py + c] = A[vo.px + c]; }
        }
    }
    std::memcpy(host_table, &h, sizeof h);
    return CTGB_OK;
}

// ---------------------------------------------------------------------------
// FDK filter tables.  Layout (float32): FilterHeader, then
//   H[zpl]        ramp spectrum in FFT order (ifftshift of Filter(...)) * deltaS / zpl
//   tw[zpl]       twiddles: cos(2 pi k / zpl), sin(2 pi k / zpl) for k < zpl/2, interleaved
//   kk[nu]        isocentre-scaled u coordinates of the cosine weight
//   pp[nv]        isocentre-scaled v coordinates of the cosine weight
namespace ctgb {
struct FilterHeader {
    int32_t zpl, log2zpl, nu, nv;
    float R;
    int32_t flip, pad[2];
    int64_t off_h, off_tw, off_kk, off_pp, total;
};

static int zero_padded_length(int nu) {
    // int(2 ** ceil(log2(2 * (nu - 1))))  (Reconstruction_numba.py:243)
    double l = std::ceil(std::log2(2.0 * (nu - 1)));
    if (nu < 2) l = 1;
    return (int)std::lround(std::pow(2.0, l));
}

static FilterHeader filter_layout(const ctgb_params *p) {
    FilterHeader f;
    std::memset(&f, 0, sizeof f);
    f.zpl = zero_padded_length(p->nu);
    f.log2zpl = 0;
    while ((1 << f.log2zpl) < f.zpl) ++f.log2zpl;
    f.nu = p->nu; f.nv = p->nv;
    int64_t off = (sizeof(FilterHeader) + 127) / 128 * 32;
    auto take = [&](int64_t n) { int64_t o = off; off += (n + 31) / 32 * 32; return o; };
    f.off_h = take(f.zpl);
    f.off_tw = take(f.zpl);
    f.off_kk = take(p->nu);
    f.off_pp = take(p->nv);
    f.total = off;
    return f;
}

// Filter(N, pixel_size, FilterType, cutoff) restated (Reconstruction_numba.py:190-225):
// spatial Ram-Lak kernel h, |fftshift(fft(h))| by a direct float64 DFT of
// length N-1, window, cutoff.  Returns the centred-order spectrum.
//   variant 0: Reconstruction.Filter — cutoff |w| > pi*cutoff/(2*tau)
//   variant 1: ConeBeam.Filter / FanBeam.Filter (python/ConeBeamGPU.py:353-379,
//              python/FanBeam.py:175-209) — spectrum doubled, cutoff |w| > pi*cutoff
//   variant 2: equiangular kernel of matlab/FilterArc.m (odd taps
//              -1/(2 pi^2 tau^2 sin^2(n tau))), cutoff as variant 0
//   variant 3: equiangular kernel of Kak & Slaney, "Principles of
//              Computerized Tomographic Imaging" eq. (3.124) (odd taps
//              -1/(2 pi^2 sin^2(n tau)), centre 1/(8 tau^2)), cutoff
//              |w| > pi*cutoff.  FilterArc.m keeps an extra tau^2 in the odd
//              taps, which unbalances the kernel for small channel angles;
//              this variant is the one that reconstructs quantitatively.
static std::vector<double> ramp_spectrum(int N, double tau, int type, double cutoff, int variant = 0) {
    const int M = N - 1;
    std::vector<double> h(M), x(N);
    for (int i = 0; i < N; ++i) x[i] = i - (N - 1) / 2.0;
    for (int i = 0; i < M; ++i) {
        double xi = x[i];
        double m = std::fmod(xi, 2.0);
        if (m < 0) m += 2.0;   // numpy's % follows the divisor's sign
        if (xi == 0) h[i] = 1.0 / (8.0 * tau * tau);
        else if (m == 1.0) {
            if (variant == 2 || variant == 3) {
                const double sn = std::sin(xi * tau);
                h[i] = -1.0 / (2.0 * M_PI * M_PI * (variant == 2 ? tau * tau : 1.0) * sn * sn);
            } else {
                h[i] = -0.5 / ((M_PI * tau * xi) * (M_PI * tau * xi));
            }
        } else h[i] = 0.0;
    }
    // |DFT(h)| then fftshift.
    std::vector<double> mag(M);
    for (int k = 0; k < M; ++k) {
        long double re = 0, im = 0;
        for (int n = 0; n < M; ++n) {
            if (h[n] == 0) continue;
            long long kn = (long long)k * n % M;
            long double a = -2.0L * M_PI * (long double)kn / M;
            re += h[n] * std::cos(a);
            im += h[n] * std::sin(a);
        }
        mag[k] = (double)std::sqrt(re * re + im * im);
    }
    std::vector<double> filt(M);
    for (int k = 0; k < M; ++k) filt[k] = mag[(k + M / 2) % M] * (variant == 1 ? 2.0 : 1.0);   // fftshift (M even)
    for (int k = 0; k < M; ++k) {
        double w = 2 * M_PI * x[k] / (N - 1);
        double f = filt[k];
        switch (type) {
            case 1:   // shepp-logan
                f = (w == 0) ? f * std::sin(w / (2.0 * cutoff)) : f * std::sin(w / (2.0 * cutoff)) / (w / (2.0 * cutoff));
                break;
            case 2: f *= std::cos(w / (2.0 * cutoff)); break;
            case 3: f *= (0.54 + 0.46 * std::cos(w / cutoff)); break;
            case 4: f *= (0.5 + 0.5 * std::cos(w / cutoff)); break;
            default: break;
        }
        const double lim = (variant == 1 || variant == 3) ? M_PI * cutoff : M_PI * cutoff / (2.0 * tau);
        if (std::fabs(w) > lim) f = 0;
        filt[k] = f;
    }
    return filt;
}
}  // namespace ctgb

extern "C" int ctgb_filter_bytes(const ctgb_params *p, size_t *bytes) {
    clear_error();
    if (!valid(p)) return last_status();
    if (p->nu < 2) return set_error(CTGB_ERR_ARG, "FDK filtering needs nu >= 2");
    if (!bytes) return set_error(CTGB_ERR_ARG, "bytes is NULL");
    FilterHeader f = filter_layout(p);
    if (f.zpl > 8192) return set_error(CTGB_ERR_SIZE, "zero-padded row length above 8192");
    *bytes = (size_t)f.total * sizeof(float);
    return CTGB_OK;
}

extern "C" int ctgb_filter_build(const ctgb_params *p, int32_t filter_type, double cutoff, void *host_buf,
                                 size_t bytes) {
    size_t need = 0;
    int st = ctgb_filter_bytes(p, &need);
    if (st != CTGB_OK) return st;
    if (!host_buf || bytes < need) return set_error(CTGB_ERR_SIZE, "filter buffer too small");
    if (filter_type < 0 || filter_type > 4) return set_error(CTGB_ERR_ARG, "unknown filter type");
    std::memset(host_buf, 0, need);
    FilterHeader f = filter_layout(p);
    Scan s = scan_of(p);
    const double R = s.sad, D = s.sdd - s.sad;
    const bool pyc = p->flavour == CTGB_FLAVOUR_PYCUDA;
    f.R = (float)R;
    float *B = static_cast<float *>(host_buf);
    const double tau = p->du * R / (D + R), delta_s = p->du * R / (R + D);
    std::vector<double> filt = ramp_spectrum(f.zpl + 1, tau, filter_type, cutoff);
    // ifftshift(filt * fftshift(X)) = ifftshift(filt) * X for even zpl.
    for (int k = 0; k < f.zpl; ++k) B[f.off_h + k] = (float)(filt[(k + f.zpl / 2) % f.zpl] * delta_s / f.zpl);
    for (int k = 0; k < f.zpl / 2; ++k) {
        B[f.off_tw + 2 * k] = (float)std::cos(2 * M_PI * k / f.zpl);
        B[f.off_tw + 2 * k + 1] = (float)std::sin(2 * M_PI * k / f.zpl);
    }
    // Filtering :229-231 (pycuda :224-227): ki, p from -n/2, scaled by R/(R+D).
    const double uoff = pyc ? p->detector_offset[0] : 0.0, voff = pyc ? p->detector_offset[1] : 0.0;
    for (int j = 0; j < p->nu; ++j) B[f.off_kk + j] = (float)(((j - p->nu / 2.0) * p->du + uoff) * R / (R + D));
    for (int i = 0; i < p->nv; ++i)
        B[f.off_pp + i] = (float)(((i - p->nv / 2.0) * (pyc ? -p->dv : p->dv) + voff) * R / (R + D));
    std::memcpy(host_buf, &f, sizeof f);
    return CTGB_OK;
}

// ---------------------------------------------------------------------------
// Standalone reconstructors' filter tables (ConeBeam / FanBeam).
static bool sa_valid(const ctgb_conebeam_params *p) {
    return p && p->source_to_axis > 0 && p->source_to_detector > p->source_to_axis && p->pixel_width > 0 &&
           p->det_width >= 2 && p->det_height >= 1 && p->nviews >= 1;
}

static FilterHeader sa_layout(const ctgb_conebeam_params *p) {
    ctgb_params q;
    std::memset(&q, 0, sizeof q);
    q.nu = p->det_width;
    q.nv = p->det_height;
    return filter_layout(&q);
}

extern "C" int ctgb_standalone_filter_bytes(const ctgb_conebeam_params *p, size_t *bytes) {
    clear_error();
    if (!sa_valid(p) || !bytes) return set_error(CTGB_ERR_ARG, "ctgb_standalone_filter_bytes: bad geometry");
    FilterHeader f = sa_layout(p);
    if (f.zpl > 8192) return set_error(CTGB_ERR_SIZE, "zero-padded row length above 8192");
    *bytes = (size_t)f.total * sizeof(float);
    return CTGB_OK;
}

// variant 0 cone beam (ConeBeamGPU.py:229-241, :298-302): weight R/sqrt(R^2+kk^2+pp^2)
//   at iso-scaled pixel centres, rows flipped along u, no deltaS;
// variant 1 fan line (FanBeam.py:111-122): weight R/sqrt(R^2+gamma^2), no deltaS;
// variant 2 fan arc (matlab/FanBeamReconArc.m:13-27): weight D*dgamma*cos(gamma),
//   arc kernel, gamma = channel angle (pitch pixel_width / SDD);
// variant 3 fan arc with the balanced equiangular kernel (same weight).
extern "C" int ctgb_standalone_filter_build(const ctgb_conebeam_params *p, int32_t variant, int32_t filter_type,
                                            double cutoff, void *host_buf, size_t bytes) {
    size_t need = 0;
    int st = ctgb_standalone_filter_bytes(p, &need);
    if (st) return st;
    if (!host_buf || bytes < need) return set_error(CTGB_ERR_SIZE, "filter buffer too small");
    if (filter_type < 0 || filter_type > 4) return set_error(CTGB_ERR_ARG, "unknown filter type");
    if (variant < 0 || variant > 3) return set_error(CTGB_ERR_ARG, "unknown filter variant");
    if (!(cutoff > 0)) return set_error(CTGB_ERR_ARG, "cutoff must be positive");
    std::memset(host_buf, 0, need);
    FilterHeader f = sa_layout(p);
    const double R = p->source_to_axis, D = p->source_to_detector - R;
    float *B = static_cast<float *>(host_buf);
    const int nu = p->det_width, nv = p->det_height;
    std::vector<double> filt;
    double scale = 1.0;
    if (variant >= 2) {
        const double dg = p->pixel_width / p->source_to_detector;   // channel angle
        filt = ramp_spectrum(f.zpl + 1, dg, filter_type, cutoff, variant);
        scale = R * dg;
        f.R = (float)R;
        for (int j = 0; j < nu; ++j) B[f.off_kk + j] = (float)(R * std::tan((j - (nu - 1) / 2.0) * dg));
        for (int i = 0; i < nv; ++i) B[f.off_pp + i] = 0.0f;
    } else {
        const double tau = p->pixel_width * R / (R + D);
        filt = ramp_spectrum(f.zpl + 1, tau, filter_type, cutoff, 1);
        f.R = (float)R;
        for (int j = 0; j < nu; ++j) B[f.off_kk + j] = (float)((j - (nu - 1) / 2.0) * tau);
        for (int i = 0; i < nv; ++i)
            B[f.off_pp + i] = variant == 0 ? (float)((i - (nv - 1) / 2.0) * p->pixel_height * R / (R + D)) : 0.0f;
        f.flip = variant == 0 ? 1 : 0;
    }
    for (int k = 0; k < f.zpl; ++k) B[f.off_h + k] = (float)(filt[(k + f.zpl / 2) % f.zpl] * scale / f.zpl);
    for (int k = 0; k < f.zpl / 2; ++k) {
        B[f.off_tw + 2 * k] = (float)std::cos(2 * M_PI * k / f.zpl);
        B[f.off_tw + 2 * k + 1] = (float)std::sin(2 * M_PI * k / f.zpl);
    }
    std::memcpy(host_buf, &f, sizeof f);
    return CTGB_OK;
}

extern "C" int ctgb_filter_zpl(const void *host_buf, int32_t *zpl) {
    clear_error();
    if (!host_buf || !zpl) return set_error(CTGB_ERR_ARG, "ctgb_filter_zpl: NULL argument");
    *zpl = static_cast<const FilterHeader *>(host_buf)->zpl;
    return CTGB_OK;
}
