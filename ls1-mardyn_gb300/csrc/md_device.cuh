// md_device.cuh -- device-side data layout and shared helpers of the engine.
//
// Layout in HBM (one context = one box):
//   master state, slot order (slots are re-sorted into list-cell order at
//   every pair-list rebuild so neighbours sit close in memory):
//     FP64 SoA  r[3] v[3] q[4] L[3] F[3] M[3] Vi[3]   (22 arrays of cap doubles)
//     int32     comp, orig (upload index), home (list cell at rebuild)
//     uint64    id
//   per-step caches:
//     float4 / double4 xl    centre position relative to the home-cell origin,
//                            .w = component index (bit pattern)
//     site cache             rotated site offsets R(q)d and orientations R(q)e
//   pair-candidate list (ELL, column-major: entry k of slot i at k*cap+i):
//     uint32  j | (cell-offset code << 27), code = (ox+1)+3(oy+1)+9(oz+1)
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define MD_MAXC 8          // components
#define MD_MAXS 8          // sites per component
#define MD_SITE_VEC 4      // elements per site record of the site caches: x, y, z and one pad (16-byte float records)
#define MD_MAXLJ 32        // LJ centres over all components
#define MD_CODE_SHIFT 27
#define MD_INDEX_MASK ((1u << MD_CODE_SHIFT) - 1u)

namespace md {

enum SiteKind : int { SK_LJ = 0, SK_CHARGE = 1, SK_DIPOLE = 2, SK_QUAD = 3 };

struct CompDev {
    int nlj, nch, ndi, nqu, ns;
    int ljoff;          // first global LJ-centre index
    int rot_dof;
    int rotates;        // any inverse inertia non-zero
    int skip_rot;       // no rotation, no torque and q a fixed point of the normalisation:
                        // the rotational half steps leave q and L unchanged and are skipped
    double m, I[3], invI[3];
    double d[MD_MAXS][3];   // body-frame site offsets, order LJ, charges, dipoles, quadrupoles
    double e[MD_MAXS][3];   // body-frame orientations (dipoles/quadrupoles)
    float df[MD_MAXS][3], ef[MD_MAXS][3];  // the same rounded to FP32 (the mixed-precision site caches)
    float If[3], invIf[3];                  // I and 1/I rounded to FP32 (mixed-precision rotational energy)
    double p[MD_MAXS];      // q, |mu| or |Q|
    int kind[MD_MAXS];
    int zero_offset[MD_MAXS];
};

struct Params {
    double bmin[3], bmax[3], L[3];
    double rc, rclj, rc2, rclj2, rlist2, epsRFInvrc3;
    int periodic[3];
    // list grid (edge >= rc + skin, no halo layer; periodic wrap)
    int ln[3];
    double lside[3], linv[3];
    // reference grid (LinkedCells: edge L/floor(L/rc), one halo layer)
    int rcpd[3];
    double rcl[3], rclr[3], rhmin[3], rhmax[3];
    int ncomp, nlj;
    int only_centred_lj;   // every component is one LJ centre at its origin
    int any_rotation;
    int max_sites;
    float rc2f, rclj2f, band_lo, band_hi, band_lo_lj, band_hi_lj;
    CompDev comp[MD_MAXC];
    double eps24[MD_MAXLJ * MD_MAXLJ], sig2[MD_MAXLJ * MD_MAXLJ], shift6[MD_MAXLJ * MD_MAXLJ];
    // FP32 copies for the mixed-precision pair kernels (no FP64 conversion per pair)
    float eps24f[MD_MAXLJ * MD_MAXLJ], sig2f[MD_MAXLJ * MD_MAXLJ], shift6f[MD_MAXLJ * MD_MAXLJ];
    float pf[MD_MAXC][MD_MAXS];
};

// parameter-table reads in the pair kernels' precision
template <typename Real> struct PTab;
template <> struct PTab<float> {
    static __device__ __forceinline__ float eps24(const Params& P, int k) { return P.eps24f[k]; }
    static __device__ __forceinline__ float sig2(const Params& P, int k) { return P.sig2f[k]; }
    static __device__ __forceinline__ float shift6(const Params& P, int k) { return P.shift6f[k]; }
    static __device__ __forceinline__ float p(const Params& P, int c, int s) { return P.pf[c][s]; }
};
template <> struct PTab<double> {
    static __device__ __forceinline__ double eps24(const Params& P, int k) { return P.eps24[k]; }
    static __device__ __forceinline__ double sig2(const Params& P, int k) { return P.sig2[k]; }
    static __device__ __forceinline__ double shift6(const Params& P, int k) { return P.shift6[k]; }
    static __device__ __forceinline__ double p(const Params& P, int c, int s) { return P.comp[c].p[s]; }
};

struct State {
    int64_t n, cap;
    double *rx, *ry, *rz, *vx, *vy, *vz, *qw, *qx, *qy, *qz, *Lx, *Ly, *Lz;
    double *Fx, *Fy, *Fz, *Mx, *My, *Mz, *Vx, *Vy, *Vz;
    int32_t *comp, *orig, *home;
    uint64_t* id;
};

// ------------------------------------------------------------------ helpers
template <typename T> struct V3 { T x, y, z; };

// Kahan-compensated accumulator (FP32 pair sums per molecule).  The
// compensation survives -use_fast_math-free compilation because nvcc does
// not reassociate floating-point additions.
struct KSum {
    float s, c;
    __device__ __forceinline__ void init() { s = 0.f; c = 0.f; }
    __device__ __forceinline__ void add(float x) {
        float y = x - c;
        float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

struct DSum {
    double s;
    __device__ __forceinline__ void init() { s = 0.0; }
    __device__ __forceinline__ void add(double x) { s += x; }
    __device__ __forceinline__ double value() const { return s; }
};

template <typename Real> struct Acc;
template <> struct Acc<float> { typedef KSum type; };
template <> struct Acc<double> { typedef DSum type; };

// Quaternion::rotate (src/molecules/Quaternion.cpp:43-64), w x y z
__device__ __forceinline__ void qrot(double w, double x, double y, double z, const double* d, double* o) {
    if (d[0] == 0.0 && d[1] == 0.0 && d[2] == 0.0) { o[0] = o[1] = o[2] = 0.0; return; }
    double ww = w * w, xx = x * x, yy = y * y, zz = z * z;
    double wx = w * x, wy = w * y, wz = w * z, xy = x * y, xz = x * z, yz = y * z;
    o[0] = (ww + xx - yy - zz) * d[0] + 2. * (xy - wz) * d[1] + 2. * (wy + xz) * d[2];
    o[1] = 2. * (wz + xy) * d[0] + (ww - xx + yy - zz) * d[1] + 2. * (yz - wx) * d[2];
    o[2] = 2. * (xz - wy) * d[0] + 2. * (wx + yz) * d[1] + (ww - xx - yy + zz) * d[2];
}

// The same rotation in FP32, for the mixed-precision site caches (the pair
// arithmetic's precision).
__device__ __forceinline__ void qrotf(float w, float x, float y, float z, const float* d, float* o) {
    if (d[0] == 0.f && d[1] == 0.f && d[2] == 0.f) { o[0] = o[1] = o[2] = 0.f; return; }
    float ww = w * w, xx = x * x, yy = y * y, zz = z * z;
    float wx = w * x, wy = w * y, wz = w * z, xy = x * y, xz = x * z, yz = y * z;
    o[0] = (ww + xx - yy - zz) * d[0] + 2.f * (xy - wz) * d[1] + 2.f * (wy + xz) * d[2];
    o[1] = 2.f * (wz + xy) * d[0] + (ww - xx + yy - zz) * d[1] + 2.f * (yz - wx) * d[2];
    o[2] = 2.f * (xz - wy) * d[0] + 2.f * (wx + yz) * d[1] + (ww - xx - yy + zz) * d[2];
}

// Quaternion::rotateinv (Quaternion.cpp:66-90)
__device__ __forceinline__ void qrotinv(double w, double x, double y, double z, const double* d, double* o) {
    if (d[0] == 0.0 && d[1] == 0.0 && d[2] == 0.0) { o[0] = o[1] = o[2] = 0.0; return; }
    double ww = w * w, xx = x * x, yy = y * y, zz = z * z;
    double wx = w * x, wy = w * y, wz = w * z, xy = x * y, xz = x * z, yz = y * z;
    o[0] = (ww + xx - yy - zz) * d[0] + 2. * (xy + wz) * d[1] + 2. * (xz - wy) * d[2];
    o[1] = 2. * (xy - wz) * d[0] + (ww - xx + yy - zz) * d[1] + 2. * (yz + wx) * d[2];
    o[2] = 2. * (xz + wy) * d[0] + 2. * (yz - wx) * d[1] + (ww - xx - yy + zz) * d[2];
}

// The inverse rotation of d by a unit quaternion (w, u) in the cross-product
// form d' = d + w t - u x t, t = -2 u x d: the rotation of qrotinv for |q| = 1
// (other rounding) in about half its FP64 operations.
__device__ __forceinline__ void qrotinv_unit(double w, double x, double y, double z, const double* d, double* o) {
    const double tx = -2. * (y * d[2] - z * d[1]);
    const double ty = -2. * (z * d[0] - x * d[2]);
    const double tz = -2. * (x * d[1] - y * d[0]);
    o[0] = d[0] + w * tx - (y * tz - z * ty);
    o[1] = d[1] + w * ty - (z * tx - x * tz);
    o[2] = d[2] + w * tz - (x * ty - y * tx);
}

// Quaternion::rotateinv in FP32 (the mixed-precision rotational energy).
__device__ __forceinline__ void qrotinvf(float w, float x, float y, float z, const float* d, float* o) {
    if (d[0] == 0.f && d[1] == 0.f && d[2] == 0.f) { o[0] = o[1] = o[2] = 0.f; return; }
    float ww = w * w, xx = x * x, yy = y * y, zz = z * z;
    float wx = w * x, wy = w * y, wz = w * z, xy = x * y, xz = x * z, yz = y * z;
    o[0] = (ww + xx - yy - zz) * d[0] + 2.f * (xy + wz) * d[1] + 2.f * (xz - wy) * d[2];
    o[1] = 2.f * (xy - wz) * d[0] + (ww - xx + yy - zz) * d[1] + 2.f * (yz + wx) * d[2];
    o[2] = 2.f * (xz + wy) * d[0] + 2.f * (yz - wx) * d[1] + (ww - xx - yy + zz) * d[2];
}

// Neighbouring doubles (IEEE successor / predecessor of a finite value), the
// std::nexttoward(r, r +- 1) of the reference's halo and leaving-particle code.
__device__ __forceinline__ double next_up(double x) {
    if (x == 0.0) return __longlong_as_double(1ll);
    long long b = __double_as_longlong(x);
    return __longlong_as_double(x > 0.0 ? b + 1 : b - 1);
}
__device__ __forceinline__ double next_down(double x) {
    if (x == 0.0) return -__longlong_as_double(1ll);
    long long b = __double_as_longlong(x);
    return __longlong_as_double(x > 0.0 ? b - 1 : b + 1);
}

__device__ __forceinline__ int decode_o(uint32_t code, int d) {
    return d == 0 ? (int)(code % 3u) - 1 : d == 1 ? (int)((code / 3u) % 3u) - 1 : (int)(code / 9u) - 1;
}

}  // namespace md
