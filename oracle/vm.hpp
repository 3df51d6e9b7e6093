// vm.hpp -- TEST INFRASTRUCTURE (oracle).  Small 3-vector / 3x3 matrix types
// whose floating-point operation order restates javax.vecmath (shipped with
// sources in the reference's jars/vecmath.jar):
//   Tuple3d.scaleAdd/interpolate/scale    Tuple3d.java:277,299,622,262
//   Vector3d.cross/normalize/dot/length   Vector3d.java:104,134,150,170
//   Point3d.distance/distanceSquared      Point3d.java:103,119
//   Matrix3d.mul/mulTransposeRight/Left   Matrix3d.java:1495,1524,1693,1737
//   Matrix3d.transform                    Matrix3d.java:2050,2064
//   Matrix3d.normalizeCP                  Matrix3d.java:1865
//   Matrix3d.invert (LU, Crout + backsub) Matrix3d.java:1045-1336
// Compile with -ffp-contract=off: Java never fuses a*b+c.
#pragma once
#include <cmath>

namespace orc {

struct V3 {
    double x = 0, y = 0, z = 0;
    V3() = default;
    V3(double a, double b, double c) : x(a), y(b), z(c) {}
    double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

inline V3 vadd(const V3& a, const V3& b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 vsub(const V3& a, const V3& b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 vscale(double s, const V3& a) { return V3(s * a.x, s * a.y, s * a.z); }
// Tuple3d.scale(double) in place: x *= s
inline void vscale_ip(V3& a, double s) { a.x *= s; a.y *= s; a.z *= s; }
// Tuple3d.scaleAdd(s, t1, t2): s*t1 + t2
inline V3 vscaleadd(double s, const V3& t1, const V3& t2) {
    return V3(s * t1.x + t2.x, s * t1.y + t2.y, s * t1.z + t2.z);
}
inline double vdot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// Vector3d.cross(v1, v2)
inline V3 vcross(const V3& v1, const V3& v2) {
    return V3(v1.y * v2.z - v1.z * v2.y, v2.x * v1.z - v2.z * v1.x, v1.x * v2.y - v1.y * v2.x);
}
inline double vlength(const V3& a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline double vlength2(const V3& a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
// Vector3d.normalize(): multiply by reciprocal of the norm
inline void vnormalize(V3& a) {
    double n = 1.0 / std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    a.x *= n; a.y *= n; a.z *= n;
}
inline double pdist(const V3& a, const V3& b) {
    double dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return std::sqrt(dx * dx + dy * dy + dz * dz);
}
inline double pdist2(const V3& a, const V3& b) {
    double dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return dx * dx + dy * dy + dz * dz;
}
// Tuple3d.interpolate(t1, t2, alpha)
inline V3 vinterp(const V3& t1, const V3& t2, double a) {
    return V3((1 - a) * t1.x + a * t2.x, (1 - a) * t1.y + a * t2.y, (1 - a) * t1.z + a * t2.z);
}

struct M3 {
    double m00 = 0, m01 = 0, m02 = 0, m10 = 0, m11 = 0, m12 = 0, m20 = 0, m21 = 0, m22 = 0;
    static M3 identity() { M3 r; r.m00 = r.m11 = r.m22 = 1; return r; }
    double get(int r, int c) const {
        const double* p = &m00; return p[3 * r + c];
    }
    void set(int r, int c, double v) { double* p = &m00; p[3 * r + c] = v; }
    V3 col(int c) const { return V3(get(0, c), get(1, c), get(2, c)); }
};

inline V3 mxv(const M3& m, const V3& t) {
    return V3(m.m00 * t.x + m.m01 * t.y + m.m02 * t.z,
              m.m10 * t.x + m.m11 * t.y + m.m12 * t.z,
              m.m20 * t.x + m.m21 * t.y + m.m22 * t.z);
}
// RigidTransform3D.inverseTransform for vectors: R^T v (RigidTransform3D.java:164-171)
inline V3 mtxv(const M3& R, const V3& v) {
    return V3(R.m00 * v.x + R.m10 * v.y + R.m20 * v.z,
              R.m01 * v.x + R.m11 * v.y + R.m21 * v.z,
              R.m02 * v.x + R.m12 * v.y + R.m22 * v.z);
}
// Matrix3d.mul(m1, m2)
inline M3 mmul(const M3& a, const M3& b) {
    M3 r;
    r.m00 = a.m00 * b.m00 + a.m01 * b.m10 + a.m02 * b.m20;
    r.m01 = a.m00 * b.m01 + a.m01 * b.m11 + a.m02 * b.m21;
    r.m02 = a.m00 * b.m02 + a.m01 * b.m12 + a.m02 * b.m22;
    r.m10 = a.m10 * b.m00 + a.m11 * b.m10 + a.m12 * b.m20;
    r.m11 = a.m10 * b.m01 + a.m11 * b.m11 + a.m12 * b.m21;
    r.m12 = a.m10 * b.m02 + a.m11 * b.m12 + a.m12 * b.m22;
    r.m20 = a.m20 * b.m00 + a.m21 * b.m10 + a.m22 * b.m20;
    r.m21 = a.m20 * b.m01 + a.m21 * b.m11 + a.m22 * b.m21;
    r.m22 = a.m20 * b.m02 + a.m21 * b.m12 + a.m22 * b.m22;
    return r;
}
// Matrix3d.mulTransposeRight(m1, m2) = m1 * m2^T
inline M3 mmulTR(const M3& a, const M3& b) {
    M3 r;
    r.m00 = a.m00 * b.m00 + a.m01 * b.m01 + a.m02 * b.m02;
    r.m01 = a.m00 * b.m10 + a.m01 * b.m11 + a.m02 * b.m12;
    r.m02 = a.m00 * b.m20 + a.m01 * b.m21 + a.m02 * b.m22;
    r.m10 = a.m10 * b.m00 + a.m11 * b.m01 + a.m12 * b.m02;
    r.m11 = a.m10 * b.m10 + a.m11 * b.m11 + a.m12 * b.m12;
    r.m12 = a.m10 * b.m20 + a.m11 * b.m21 + a.m12 * b.m22;
    r.m20 = a.m20 * b.m00 + a.m21 * b.m01 + a.m22 * b.m02;
    r.m21 = a.m20 * b.m10 + a.m21 * b.m11 + a.m22 * b.m12;
    r.m22 = a.m20 * b.m20 + a.m21 * b.m21 + a.m22 * b.m22;
    return r;
}
// Matrix3d.mulTransposeLeft(m1, m2) = m1^T * m2
inline M3 mmulTL(const M3& a, const M3& b) {
    M3 r;
    r.m00 = a.m00 * b.m00 + a.m10 * b.m10 + a.m20 * b.m20;
    r.m01 = a.m00 * b.m01 + a.m10 * b.m11 + a.m20 * b.m21;
    r.m02 = a.m00 * b.m02 + a.m10 * b.m12 + a.m20 * b.m22;
    r.m10 = a.m01 * b.m00 + a.m11 * b.m10 + a.m21 * b.m20;
    r.m11 = a.m01 * b.m01 + a.m11 * b.m11 + a.m21 * b.m21;
    r.m12 = a.m01 * b.m02 + a.m11 * b.m12 + a.m21 * b.m22;
    r.m20 = a.m02 * b.m00 + a.m12 * b.m10 + a.m22 * b.m20;
    r.m21 = a.m02 * b.m01 + a.m12 * b.m11 + a.m22 * b.m21;
    r.m22 = a.m02 * b.m02 + a.m12 * b.m12 + a.m22 * b.m22;
    return r;
}
inline M3 madd(const M3& a, const M3& b) {
    M3 r; const double* pa = &a.m00; const double* pb = &b.m00; double* pr = &r.m00;
    for (int i = 0; i < 9; i++) pr[i] = pa[i] + pb[i];
    return r;
}
inline M3 msub(const M3& a, const M3& b) {
    M3 r; const double* pa = &a.m00; const double* pb = &b.m00; double* pr = &r.m00;
    for (int i = 0; i < 9; i++) pr[i] = pa[i] - pb[i];
    return r;
}
inline M3 mscale(const M3& a, double s) {  // Matrix3d.mul(double): m *= s
    M3 r; const double* pa = &a.m00; double* pr = &r.m00;
    for (int i = 0; i < 9; i++) pr[i] = pa[i] * s;
    return r;
}
// Matrix3d.normalizeCP(m1)
inline M3 mnormalizeCP(const M3& m1) {
    M3 r;
    double mag = 1.0 / std::sqrt(m1.m00 * m1.m00 + m1.m10 * m1.m10 + m1.m20 * m1.m20);
    r.m00 = m1.m00 * mag; r.m10 = m1.m10 * mag; r.m20 = m1.m20 * mag;
    mag = 1.0 / std::sqrt(m1.m01 * m1.m01 + m1.m11 * m1.m11 + m1.m21 * m1.m21);
    r.m01 = m1.m01 * mag; r.m11 = m1.m11 * mag; r.m21 = m1.m21 * mag;
    r.m02 = r.m10 * r.m21 - r.m11 * r.m20;
    r.m12 = r.m01 * r.m20 - r.m00 * r.m21;
    r.m22 = r.m00 * r.m11 - r.m01 * r.m10;
    return r;
}

// Matrix3d.invertGeneral: Crout LU with implicit row scaling, then back
// substitution on the identity.  Returns false when singular.
inline bool minvert(const M3& m1, M3& out) {
    double t[9] = {m1.m00, m1.m01, m1.m02, m1.m10, m1.m11, m1.m12, m1.m20, m1.m21, m1.m22};
    int perm[3];
    double scale[3];
    {
        int ptr = 0, rs = 0;
        for (int i = 3; i-- != 0;) {
            double big = 0.0;
            for (int j = 3; j-- != 0;) {
                double tmp = std::fabs(t[ptr++]);
                if (tmp > big) big = tmp;
            }
            if (big == 0.0) return false;
            scale[rs++] = 1.0 / big;
        }
    }
    for (int j = 0; j < 3; j++) {
        for (int i = 0; i < j; i++) {
            int target = 3 * i + j;
            double sum = t[target];
            int p1 = 3 * i, p2 = j;
            for (int k = i; k-- != 0;) { sum -= t[p1] * t[p2]; p1++; p2 += 3; }
            t[target] = sum;
        }
        double big = 0.0;
        int imax = -1;
        for (int i = j; i < 3; i++) {
            int target = 3 * i + j;
            double sum = t[target];
            int p1 = 3 * i, p2 = j;
            for (int k = j; k-- != 0;) { sum -= t[p1] * t[p2]; p1++; p2 += 3; }
            t[target] = sum;
            double tmp = scale[i] * std::fabs(sum);
            if (tmp >= big) { big = tmp; imax = i; }
        }
        if (imax < 0) return false;
        if (j != imax) {
            int p1 = 3 * imax, p2 = 3 * j;
            for (int k = 3; k-- != 0;) { double tmp = t[p1]; t[p1++] = t[p2]; t[p2++] = tmp; }
            scale[imax] = scale[j];
        }
        perm[j] = imax;
        if (t[3 * j + j] == 0.0) return false;
        if (j != 2) {
            double tmp = 1.0 / t[3 * j + j];
            int target = 3 * (j + 1) + j;
            for (int i = 2 - j; i-- != 0;) { t[target] *= tmp; target += 3; }
        }
    }
    double r[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int k = 0; k < 3; k++) {
        int cv = k, ii = -1;
        for (int i = 0; i < 3; i++) {
            int ip = perm[i];
            double sum = r[cv + 3 * ip];
            r[cv + 3 * ip] = r[cv + 3 * i];
            if (ii >= 0) {
                int rv = i * 3;
                for (int j = ii; j <= i - 1; j++) sum -= t[rv + j] * r[cv + 3 * j];
            } else if (sum != 0.0) {
                ii = i;
            }
            r[cv + 3 * i] = sum;
        }
        int rv = 6;
        r[cv + 6] /= t[rv + 2];
        rv -= 3;
        r[cv + 3] = (r[cv + 3] - t[rv + 2] * r[cv + 6]) / t[rv + 1];
        rv -= 3;
        r[cv + 0] = (r[cv + 0] - t[rv + 1] * r[cv + 3] - t[rv + 2] * r[cv + 6]) / t[rv + 0];
    }
    out.m00 = r[0]; out.m01 = r[1]; out.m02 = r[2];
    out.m10 = r[3]; out.m11 = r[4]; out.m12 = r[5];
    out.m20 = r[6]; out.m21 = r[7]; out.m22 = r[8];
    return true;
}

// Rigid transform (R, t) as RigidTransform3D.java restates it.
struct RT {
    M3 R; V3 t;
};
inline V3 rt_point(const RT& T, const V3& p) { return vadd(mxv(T.R, p), T.t); }    // transform(Point3d)
inline V3 rt_vec(const RT& T, const V3& v) { return mxv(T.R, v); }                 // transform(Vector3d)
inline V3 rt_inv_point(const RT& T, const V3& p) {                                  // inverseTransform(Point3d)
    double x = p.x - T.t.x, y = p.y - T.t.y, z = p.z - T.t.z;
    return V3(T.R.m00 * x + T.R.m10 * y + T.R.m20 * z,
              T.R.m01 * x + T.R.m11 * y + T.R.m21 * z,
              T.R.m02 * x + T.R.m12 * y + T.R.m22 * z);
}
// RigidTransform3D.mult(A, B): this = A*B  (t = A.R*B.t + A.t ; R = A.R*B.R)
inline RT rt_mult(const RT& A, const RT& B) {
    RT r; r.t = vadd(mxv(A.R, B.t), A.t); r.R = mmul(A.R, B.R); return r;
}
// RigidTransform3D.multAinvB(A, B): t = A.R^T (B.t - A.t); R = A.R^T B.R
inline RT rt_multAinvB(const RT& A, const RT& B) {
    RT r;
    V3 t = vsub(B.t, A.t);
    M3 RT_ = M3();
    RT_.m00 = A.R.m00; RT_.m01 = A.R.m10; RT_.m02 = A.R.m20;
    RT_.m10 = A.R.m01; RT_.m11 = A.R.m11; RT_.m12 = A.R.m21;
    RT_.m20 = A.R.m02; RT_.m21 = A.R.m12; RT_.m22 = A.R.m22;
    r.t = mxv(RT_, t);
    r.R = mmul(RT_, B.R);
    return r;
}
// RigidTransform3D.computeRM0RT: M2 = R M1 R^T
inline M3 rm0rt(const M3& R, const M3& M1) { return mmulTR(mmul(R, M1), R); }
// RigidTransform3D.computeRTMR: M2 = R^T M1 R
inline M3 rtmr(const M3& R, const M3& M1) { return mmul(mmulTL(R, M1), R); }

}  // namespace orc
