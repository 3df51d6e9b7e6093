// am_dev.cuh -- device-side 3-vector / 3x3 helpers for the FP64 drop-in.
//
// Every helper evaluates in the operation order of javax.vecmath (the
// reference's math library): Matrix3d.transform = row dot products summed
// left to right, Vector3d.cross, Tuple3d.scaleAdd (s*t1 + t2), Matrix3d.mul,
// Matrix3d.normalizeCP, Matrix3d.invert (Crout LU).  The translation units
// that include this header are compiled with --fmad=false so that no a*b+c is
// contracted, which is what makes the device results bit-identical to the
// reference arithmetic.
#pragma once
#include <cstdint>
#include <cstring>

namespace amd {

struct v3 { double x, y, z; };

__host__ __device__ __forceinline__ v3 mk(double x, double y, double z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
__host__ __device__ __forceinline__ v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ v3 scale(double s, v3 a) { return mk(s * a.x, s * a.y, s * a.z); }
__host__ __device__ __forceinline__ v3 scaleadd(double s, v3 t1, v3 t2) { return mk(s * t1.x + t2.x, s * t1.y + t2.y, s * t1.z + t2.z); }
__host__ __device__ __forceinline__ double dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ v3 cross(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, b.x * a.z - b.z * a.x, a.x * b.y - a.y * b.x);
}
__host__ __device__ __forceinline__ double length(v3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
__host__ __device__ __forceinline__ void normalize(v3& a) {
    double n = 1.0 / sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    a.x *= n; a.y *= n; a.z *= n;
}
__host__ __device__ __forceinline__ double dist(v3 a, v3 b) {
    double dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return sqrt(dx * dx + dy * dy + dz * dz);
}
__host__ __device__ __forceinline__ double dist2(v3 a, v3 b) {
    double dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return dx * dx + dy * dy + dz * dz;
}
__host__ __device__ __forceinline__ double comp(v3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
__host__ __device__ __forceinline__ void setc(v3& a, int i, double v) { if (i == 0) a.x = v; else if (i == 1) a.y = v; else a.z = v; }

// 3x3 row-major in 9 consecutive doubles
struct m3 { double m[9]; };

__host__ __device__ __forceinline__ m3 ldm(const double* p) { m3 r; for (int k = 0; k < 9; k++) r.m[k] = p[k]; return r; }
__host__ __device__ __forceinline__ void stm(double* p, const m3& a) { for (int k = 0; k < 9; k++) p[k] = a.m[k]; }
__host__ __device__ __forceinline__ v3 ldv(const double* p) { return mk(p[0], p[1], p[2]); }
__host__ __device__ __forceinline__ void stv(double* p, v3 a) { p[0] = a.x; p[1] = a.y; p[2] = a.z; }
__host__ __device__ __forceinline__ m3 ident() { m3 r; for (int k = 0; k < 9; k++) r.m[k] = (k % 4 == 0) ? 1.0 : 0.0; return r; }
__host__ __device__ __forceinline__ m3 zero3() { m3 r; for (int k = 0; k < 9; k++) r.m[k] = 0.0; return r; }
__host__ __device__ __forceinline__ v3 col(const m3& a, int c) { return mk(a.m[c], a.m[3 + c], a.m[6 + c]); }

// Matrix3d.transform(t)
__host__ __device__ __forceinline__ v3 mxv(const m3& a, v3 t) {
    return mk(a.m[0] * t.x + a.m[1] * t.y + a.m[2] * t.z,
              a.m[3] * t.x + a.m[4] * t.y + a.m[5] * t.z,
              a.m[6] * t.x + a.m[7] * t.y + a.m[8] * t.z);
}
// R^T v, as RigidTransform3D.inverseTransform writes it
__host__ __device__ __forceinline__ v3 mtxv(const m3& R, v3 v) {
    return mk(R.m[0] * v.x + R.m[3] * v.y + R.m[6] * v.z,
              R.m[1] * v.x + R.m[4] * v.y + R.m[7] * v.z,
              R.m[2] * v.x + R.m[5] * v.y + R.m[8] * v.z);
}
// Matrix3d.mul(a, b)
__host__ __device__ __forceinline__ m3 mmul(const m3& a, const m3& b) {
    m3 r;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            r.m[3 * i + j] = a.m[3 * i] * b.m[j] + a.m[3 * i + 1] * b.m[3 + j] + a.m[3 * i + 2] * b.m[6 + j];
    return r;
}
// Matrix3d.mulTransposeRight(a, b) = a b^T
__host__ __device__ __forceinline__ m3 mmulTR(const m3& a, const m3& b) {
    m3 r;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            r.m[3 * i + j] = a.m[3 * i] * b.m[3 * j] + a.m[3 * i + 1] * b.m[3 * j + 1] + a.m[3 * i + 2] * b.m[3 * j + 2];
    return r;
}
// Matrix3d.mulTransposeLeft(a, b) = a^T b
__host__ __device__ __forceinline__ m3 mmulTL(const m3& a, const m3& b) {
    m3 r;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            r.m[3 * i + j] = a.m[i] * b.m[j] + a.m[3 + i] * b.m[3 + j] + a.m[6 + i] * b.m[6 + j];
    return r;
}
// RigidTransform3D.computeRM0RT: R M R^T
__host__ __device__ __forceinline__ m3 rm0rt(const m3& R, const m3& M) { return mmulTR(mmul(R, M), R); }
// RigidTransform3D.computeRTMR: R^T M R
__host__ __device__ __forceinline__ m3 rtmr(const m3& R, const m3& M) { return mmul(mmulTL(R, M), R); }

// Matrix3d.normalizeCP
__host__ __device__ __forceinline__ m3 normalizeCP(const m3& a) {
    m3 r;
    double mag = 1.0 / sqrt(a.m[0] * a.m[0] + a.m[3] * a.m[3] + a.m[6] * a.m[6]);
    r.m[0] = a.m[0] * mag; r.m[3] = a.m[3] * mag; r.m[6] = a.m[6] * mag;
    mag = 1.0 / sqrt(a.m[1] * a.m[1] + a.m[4] * a.m[4] + a.m[7] * a.m[7]);
    r.m[1] = a.m[1] * mag; r.m[4] = a.m[4] * mag; r.m[7] = a.m[7] * mag;
    r.m[2] = r.m[3] * r.m[7] - r.m[4] * r.m[6];
    r.m[5] = r.m[1] * r.m[6] - r.m[0] * r.m[7];
    r.m[8] = r.m[0] * r.m[4] - r.m[1] * r.m[3];
    return r;
}

// Matrix3d.invert: Crout LU with implicit row scaling and partial pivoting,
// then back substitution on the identity (the algorithm of javax.vecmath's
// Matrix3d.invertGeneral / luDecomposition / luBacksubstitution, written out
// in the same operation order).  Returns false for a singular matrix.
__host__ __device__ inline bool invert3(const m3& a, m3& out) {
    double t[9];
    for (int k = 0; k < 9; k++) t[k] = a.m[k];
    int perm[3];
    double scl[3];
    for (int i = 0, ptr = 0; i < 3; i++) {
        double big = 0.0;
        for (int j = 0; j < 3; j++) { double v = fabs(t[ptr++]); if (v > big) big = v; }
        if (big == 0.0) return false;
        scl[i] = 1.0 / big;
    }
    for (int j = 0; j < 3; j++) {
        for (int i = 0; i < j; i++) {
            double sum = t[3 * i + j];
            for (int k = 0; k < i; k++) sum -= t[3 * i + k] * t[3 * k + j];
            t[3 * i + j] = sum;
        }
        double big = 0.0;
        int imax = -1;
        for (int i = j; i < 3; i++) {
            double sum = t[3 * i + j];
            for (int k = 0; k < j; k++) sum -= t[3 * i + k] * t[3 * k + j];
            t[3 * i + j] = sum;
            double v = scl[i] * fabs(sum);
            if (v >= big) { big = v; imax = i; }
        }
        if (imax < 0) return false;
        if (j != imax) {
            for (int k = 0; k < 3; k++) { double v = t[3 * imax + k]; t[3 * imax + k] = t[3 * j + k]; t[3 * j + k] = v; }
            scl[imax] = scl[j];
        }
        perm[j] = imax;
        if (t[3 * j + j] == 0.0) return false;
        if (j != 2) {
            double v = 1.0 / t[3 * j + j];
            for (int i = j + 1; i < 3; i++) t[3 * i + j] *= v;
        }
    }
    double r[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int k = 0; k < 3; k++) {
        int ii = -1;
        for (int i = 0; i < 3; i++) {
            int ip = perm[i];
            double sum = r[k + 3 * ip];
            r[k + 3 * ip] = r[k + 3 * i];
            if (ii >= 0) {
                for (int j = ii; j <= i - 1; j++) sum -= t[3 * i + j] * r[k + 3 * j];
            } else if (sum != 0.0) {
                ii = i;
            }
            r[k + 3 * i] = sum;
        }
        r[k + 6] /= t[8];
        r[k + 3] = (r[k + 3] - t[5] * r[k + 6]) / t[4];
        r[k] = (r[k] - t[1] * r[k + 3] - t[2] * r[k + 6]) / t[0];
    }
    for (int q = 0; q < 9; q++) out.m[q] = r[q];
    return true;
}

// rigid transform helpers: T = (R, t)
__host__ __device__ __forceinline__ v3 tpoint(const m3& R, v3 t, v3 p) { return add(mxv(R, p), t); }
__host__ __device__ __forceinline__ v3 tinvpoint(const m3& R, v3 t, v3 p) {
    double x = p.x - t.x, y = p.y - t.y, z = p.z - t.z;
    return mk(R.m[0] * x + R.m[3] * y + R.m[6] * z,
              R.m[1] * x + R.m[4] * y + R.m[7] * z,
              R.m[2] * x + R.m[5] * y + R.m[8] * z);
}

// java.lang.Math.max / min semantics (NaN first argument, signed zeros)
__host__ __device__ __forceinline__ double jmax(double a, double b) {
    if (a != a) return a;
    if (a == 0.0 && b == 0.0 && signbit(a)) return b;
    return (a >= b) ? a : b;
}
__host__ __device__ __forceinline__ double jmin(double a, double b) {
    if (a != a) return a;
    if (a == 0.0 && b == 0.0 && signbit(b)) return b;
    return (a <= b) ? a : b;
}

// The same Math.max / Math.min on IEEE bit patterns, for the sweeps where
// every FP64 instruction costs a full pass of the FP64 pipe: a NaN test on
// the bits, then an integer comparison of keys that order non-NaN doubles as
// their values do (the bits for a positive sign, the bits with the magnitude
// inverted for a negative one, so -0 < +0).  The results are the same bits as
// jmax / jmin for every pair of arguments.
__host__ __device__ __forceinline__ long long dbits(double x) {
#ifdef __CUDA_ARCH__
    return __double_as_longlong(x);
#else
    long long b;
    std::memcpy(&b, &x, sizeof b);
    return b;
#endif
}
__host__ __device__ __forceinline__ double dfrombits(long long b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double(b);
#else
    double x;
    std::memcpy(&x, &b, sizeof x);
    return x;
#endif
}
__host__ __device__ __forceinline__ bool nan_bits(long long b) {
    return (b & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
}
__host__ __device__ __forceinline__ long long order_key(long long b) { return b < 0 ? b ^ 0x7fffffffffffffffll : b; }
__host__ __device__ __forceinline__ double jmax_i(double a, double b) {
    const long long x = dbits(a), y = dbits(b);
    if (nan_bits(x)) return a;
    if (nan_bits(y)) return b;
    return order_key(x) >= order_key(y) ? a : b;
}
__host__ __device__ __forceinline__ double jmin_i(double a, double b) {
    const long long x = dbits(a), y = dbits(b);
    if (nan_bits(x)) return a;
    if (nan_bits(y)) return b;
    return order_key(x) <= order_key(y) ? a : b;
}
// |a| and -a by the sign bit (the same bits as fabs and unary minus)
__host__ __device__ __forceinline__ double abs_i(double a) { return dfrombits(dbits(a) & 0x7fffffffffffffffll); }
__host__ __device__ __forceinline__ double neg_i(double a) {
    return dfrombits(dbits(a) ^ (long long)0x8000000000000000ull);
}

// Deterministic sine/cosine for the Rodrigues rotation update: Cody-Waite
// reduction by pi/2 (two-term constant, C1 = pi/2 to 33 bits) and Taylor
// series on |r| <= pi/4 (sin to r^17, cos to r^18), Horner in r^2.  The same
// published method, in the same operation order, is used by the CPU restatement,
// so both produce identical bits.  Valid for 0 <= x < 2^20.
__host__ __device__ __forceinline__ void det_sincos(double x, double* s_out, double* c_out) {
    const double TWO_OVER_PI = 0.6366197723675814;
    const double C1 = 1.5707963267341256;
    const double C2 = 6.077100506506192e-11;
    double k = floor(x * TWO_OVER_PI + 0.5);
    double r = (x - k * C1) - k * C2;
    double z = r * r;
    double ps = 2.8114572543455206e-15;
    ps = -7.647163731819816e-13 + z * ps;
    ps = 1.6059043836821613e-10 + z * ps;
    ps = -2.505210838544172e-08 + z * ps;
    ps = 2.7557319223985893e-06 + z * ps;
    ps = -1.984126984126984e-04 + z * ps;
    ps = 8.333333333333333e-03 + z * ps;
    ps = -1.6666666666666666e-01 + z * ps;
    double sr = r + (r * z) * ps;
    double pc = -1.5619206968586225e-16;
    pc = 4.779477332387385e-14 + z * pc;
    pc = -1.1470745597729725e-11 + z * pc;
    pc = 2.08767569878681e-09 + z * pc;
    pc = -2.755731922398589e-07 + z * pc;
    pc = 2.48015873015873e-05 + z * pc;
    pc = -1.388888888888889e-03 + z * pc;
    pc = 4.1666666666666664e-02 + z * pc;
    double cr = (1.0 - 0.5 * z) + (z * z) * pc;
    long long q = (long long)k & 3;
    if (q == 0) { *s_out = sr; *c_out = cr; }
    else if (q == 1) { *s_out = cr; *c_out = -sr; }
    else if (q == 2) { *s_out = -sr; *c_out = -cr; }
    else { *s_out = -cr; *c_out = sr; }
}

}  // namespace amd
