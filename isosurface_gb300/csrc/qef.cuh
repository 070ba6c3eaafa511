// Feature placement for DualContouring (and, through the row-bounded SVD
// steps, ExtendedMarchingCubes), on the device and on the host.
//
// * TangentPlanes::new over the 8 cell corners (src/feature/mod.rs:91-148)
//   and ParticleBasedMinimisation (src/feature/particle_minimisation.rs:25-72),
//   the f32 half, in qef_planes.cuh
// * MinimiseQEF (src/feature/qef.rs:36-68) with the 3-column f64 SVD of
//   src/math/svd.rs: Householder bidiagonalisation (factorize, :149-292),
//   accumulation of U and V (unpack, :295-410), implicit-shift QR with Givens
//   rotations (diagonalize/qrstep*, :413-847), sign and order normalisation
//   (singularize, :892-925) and the truncated solve (SVD::solve + solveSVD,
//   :55-84, :928-972: singular values below 0.1 are zeroed and then skipped,
//   which leaves their projection in the solution unscaled).
//
// The SVD steps are restated from swiftcoder/isosurface (src/math/svd.rs),
// Copyright 2021 Tristam MacDonald, licensed under the Apache License, Version
// 2.0 (http://www.apache.org/licenses/LICENSE-2.0).
//
// The steps and their operation order follow the reference so that vertex
// positions match it bit for bit (the translation unit is built with
// -fmad=false; f64 sqrt and division are IEEE).  The reference's QR loop has
// no iteration bound; here it stops after QR_SWEEP_LIMIT sweeps and reports it.
#pragma once
#include <cuda_runtime.h>

#include "qef_planes.cuh"

namespace iso {
namespace qef {

constexpr int QR_SWEEP_LIMIT = 10000;

// factorize_hh
__host__ __device__ inline double householder(double** x, int n) {
    double tau = 0.0;
    if (n > 1) {
        double xnorm;
        if (n == 2) {
            xnorm = fabs(*x[1]);
        } else {
            double scl = 0.0, ssq = 1.0;
            for (int i = 1; i < n; ++i) {
                const double v = fabs(*x[i]);
                if (v != 0.0) {
                    if (scl < v) {
                        ssq = 1.0 + ssq * (scl / v) * (scl / v);
                        scl = v;
                    } else {
                        ssq += v / scl * (v / scl);
                    }
                }
            }
            xnorm = scl * sqrt(ssq);
        }
        if (xnorm != 0.0) {
            const double alpha = *x[0];
            double beta = sqrt(alpha * alpha + xnorm * xnorm);
            if (alpha >= 0.0) beta = -beta;
            tau = (beta - alpha) / beta;
            const double s = 1.0 / (alpha - beta);
            *x[0] = beta;
            for (int i = 1; i < n; ++i) *x[i] *= s;
        }
    }
    return tau;
}

// R bounds `rows` (8 for DualContouring's corners, 12 for the edge crossings
// of ExtendedMarchingCubes)
template <int R = 8>
__host__ __device__ inline void bidiagonalise(double (*m)[3], double* tau_u, double* tau_v, int rows) {
    for (int i = 0; i < 3; ++i) {
        double* col[R];
        const int n = rows - i;
        for (int q = 0; q < n; ++q) col[q] = &m[q + i][i];
        double tau = householder(col, n);
        tau_u[i] = tau;
        if (i + 1 < 3) {
            if (tau != 0.0) {
                for (int x = i + 1; x < 3; ++x) {
                    double wx = m[i][x];
                    for (int y = i + 1; y < rows; ++y) wx += m[y][x] * *col[y - i];
                    const double tau_wx = tau * wx;
                    m[i][x] -= tau_wx;
                    for (int y = i + 1; y < rows; ++y) m[y][x] -= tau_wx * *col[y - i];
                }
            }
            double* row[2];
            row[0] = &m[i][i + 1];
            int nr = 1;
            if (i == 0) {
                row[1] = &m[i][i + 2];
                nr = 2;
            }
            tau = householder(row, nr);
            tau_v[i] = tau;
            if (tau != 0.0) {
                for (int y = i + 1; y < rows; ++y) {
                    double wy = m[y][i + 1];
                    if (i == 0) wy += m[y][i + 2] * *row[1];
                    const double tau_wy = tau * wy;
                    m[y][i + 1] -= tau_wy;
                    if (i == 0) m[y][i + 2] -= tau_wy * *row[1];
                }
            }
        }
    }
}

__host__ __device__ inline void unpack(double (*u)[3], double (*v)[3], double* tau_u, double* tau_v, int rows) {
    v[0][0] = v[1][1] = v[2][2] = 1.0;
    v[0][1] = v[0][2] = v[1][0] = v[1][2] = v[2][0] = v[2][1] = 0.0;
    for (int i = 1; i >= 0; --i) {
        const double tau = tau_v[i];
        if (tau != 0.0) {
            for (int x = i + 1; x < 3; ++x) {
                double wx = v[i + 1][x];
                for (int y = i + 2; y < 3; ++y) wx += v[y][x] * u[i][y];
                const double tau_wx = tau * wx;
                v[i + 1][x] -= tau_wx;
                for (int y = i + 2; y < 3; ++y) v[y][x] -= tau_wx * u[i][y];
            }
        }
    }
    for (int i = 0; i < 2; ++i) tau_v[i] = u[i][i + 1];
    for (int i = 2; i >= 0; --i) {
        const double tau = tau_u[i];
        tau_u[i] = u[i][i];
        if (tau == 0.0) {
            u[i][i] = 1.0;
            if (i < 2) {
                u[i][2] = 0.0;
                if (i < 1) u[i][1] = 0.0;
            }
            for (int y = i + 1; y < rows; ++y) u[y][i] = 0.0;
        } else {
            for (int x = i + 1; x < 3; ++x) {
                double wx = 0.0;
                for (int y = i + 1; y < rows; ++y) wx += u[y][x] * u[y][i];
                const double tau_wx = tau * wx;
                u[i][x] = -tau_wx;
                for (int y = i + 1; y < rows; ++y) u[y][x] -= tau_wx * u[y][i];
            }
            for (int y = i + 1; y < rows; ++y) u[y][i] = u[y][i] * -tau;
            u[i][i] = 1.0 - tau;
        }
    }
}

__host__ __device__ inline void chop(double* a, double* b, int n) {
    double ai = a[0];
    for (int i = 0; i < n - 1; ++i) {
        const double bi = b[i];
        const double ai1 = a[i + 1];
        if (fabs(bi) < 1e-5 * (fabs(ai) + fabs(ai1))) b[i] = 0.0;
        ai = ai1;
    }
}

__host__ __device__ inline void givens(double a, double b, double* c, double* s) {
    if (b == 0.0) {
        *c = 1.0;
        *s = 0.0;
    } else if (fabs(b) > fabs(a)) {
        const double t = -a / b;
        const double s1 = 1.0 / sqrt(1.0 + t * t);
        *s = s1;
        *c = s1 * t;
    } else {
        const double t = -b / a;
        const double c1 = 1.0 / sqrt(1.0 + t * t);
        *c = c1;
        *s = c1 * t;
    }
}

__host__ __device__ inline void schur(double a1, double a2, double a3, double* c, double* s) {
    const double apq = a1 * a2 * 2.0;
    if (apq == 0.0) {
        *c = 1.0;
        *s = 0.0;
    } else {
        double t;
        const double tau = (a2 * a2 + (a3 + a1) * (a3 - a1)) / apq;
        if (tau >= 0.0) t = 1.0 / (tau + sqrt(1.0 + tau * tau));
        else t = -1.0 / (sqrt(1.0 + tau * tau) - tau);
        *c = 1.0 / sqrt(1.0 + t * t);
        *s = t * *c;
    }
}

__host__ __device__ __forceinline__ void rot_cols(double (*m)[3], int rows, int p, int q, double c, double s) {
    for (int i = 0; i < rows; ++i) {
        const double mp = m[i][p], mq = m[i][q];
        m[i][p] = mp * c - mq * s;
        m[i][q] = mp * s + mq * c;
    }
}

__host__ __device__ inline void qr_middle(double (*u)[3], double* tau_u, double* tau_v, int rows, int cols, int col) {
    double x = tau_v[col];
    double y = tau_u[col + 1];
    for (int j = col; j < cols - 1; ++j) {
        double c, s;
        givens(y, -x, &c, &s);
        for (int i = 0; i < rows; ++i) {
            const double up = u[i][col], uq = u[i][j + 1];
            u[i][col] = up * c - uq * s;
            u[i][j + 1] = up * s + uq * c;
        }
        tau_u[j + 1] = x * s + y * c;
        if (j == col) tau_v[j] = x * c - y * s;
        if (j < cols - 2) {
            const double z = tau_v[j + 1];
            tau_v[j + 1] *= c;
            x = z * -s;
            y = tau_u[j + 2];
        }
    }
}

__host__ __device__ inline void qr_end(double (*v)[3], double* tau_u, double* tau_v) {
    double x = tau_u[1];
    double y = tau_v[1];
    for (int k = 1; k >= 0; --k) {
        double c, s;
        givens(x, y, &c, &s);
        rot_cols(v, 3, k, 2, c, s);
        tau_u[k] = x * c - y * s;
        if (k == 1) tau_v[k] = x * s + y * c;
        if (k > 0) {
            const double z = tau_v[k - 1];
            tau_v[k - 1] *= c;
            x = tau_u[k - 1];
            y = z * s;
        }
    }
}

__host__ __device__ inline double shift(const double* tau_u, const double* tau_v) {
    const double ta = tau_u[1] * tau_u[1] + tau_v[0] * tau_v[0];
    const double tb = tau_u[2] * tau_u[2] + tau_v[1] * tau_v[1];
    const double tab = tau_u[1] * tau_v[1];
    const double dt = (ta - tb) / 2.0;
    if (dt >= 0.0) return tb - tab * tab / (dt + sqrt(dt * dt + tab * tab));
    return tb + tab * tab / (sqrt(dt * dt + tab * tab) - dt);
}

__host__ __device__ inline void qr_cols2(double (*u)[3], double (*v)[3], double* tau_u, double* tau_v, int rows) {
    if (tau_u[0] == 0.0) {
        double c, s;
        givens(tau_v[0], tau_u[1], &c, &s);
        tau_u[0] = tau_v[0] * c - tau_u[1] * s;
        tau_v[0] = tau_v[0] * s + tau_u[1] * c;
        tau_u[1] = 0.0;
        rot_cols(u, rows, 0, 1, c, s);
        for (int i = 0; i < 3; ++i) {
            const double t = v[i][0];
            v[i][0] = v[i][1];
            v[i][1] = t;
        }
    } else if (tau_u[1] == 0.0) {
        double c, s;
        givens(tau_u[0], tau_v[0], &c, &s);
        tau_u[0] = tau_u[0] * c - tau_v[0] * s;
        tau_v[0] = 0.0;
        rot_cols(v, 3, 0, 1, c, s);
    } else {
        double c, s;
        schur(tau_u[0], tau_v[0], tau_u[1], &c, &s);
        double a11 = tau_u[0] * c - tau_v[0] * s;
        double a21 = -tau_u[1] * s;
        double a12 = tau_u[0] * s + tau_v[0] * c;
        double a22 = tau_u[1] * c;
        rot_cols(v, 3, 0, 1, c, s);
        if (a11 * a11 + a21 * a21 < a12 * a12 + a22 * a22) {
            double t = a11;
            a11 = a12;
            a12 = t;
            t = a21;
            a21 = a22;
            a22 = t;
            for (int i = 0; i < 3; ++i) {
                t = v[i][0];
                v[i][0] = v[i][1];
                v[i][1] = t;
            }
        }
        givens(a11, a21, &c, &s);
        tau_u[0] = a11 * c - a21 * s;
        tau_v[0] = a12 * c - a22 * s;
        tau_u[1] = a12 * s + a22 * c;
        rot_cols(u, rows, 0, 1, c, s);
    }
}

__host__ __device__ inline void qr_step(double (*u)[3], double (*v)[3], double* tau_u, double* tau_v, int rows, int cols) {
    if (cols == 2) {
        qr_cols2(u, v, tau_u, tau_v, rows);
        return;
    }
    for (int i = 0; i < cols - 1; ++i) {
        if (tau_u[i] == 0.0) {
            qr_middle(u, tau_u, tau_v, rows, cols, i);
            return;
        }
    }
    if (tau_u[cols - 1] == 0.0) {
        qr_end(v, tau_u, tau_v);
        return;
    }
    const double mu = shift(tau_u, tau_v);
    double y = tau_u[0] * tau_u[0] - mu;
    double z = tau_u[0] * tau_v[0];
    double ak = 0.0, bk = 0.0, zk;
    double ap = tau_u[0], bp = tau_v[0], aq = tau_u[1];
    for (int k = 0; k < cols - 1; ++k) {
        double c, s;
        givens(y, z, &c, &s);
        rot_cols(v, 3, k, k + 1, c, s);
        double bk1 = bk * c - z * s;
        double ap1 = ap * c - bp * s;
        double bp1 = ap * s + bp * c;
        const double zp1 = aq * -s;
        const double aq1 = aq * c;
        if (k > 0) tau_v[k - 1] = bk1;
        ak = ap1;
        bk = bp1;
        zk = zp1;
        ap = aq1;
        bp = (k < cols - 2) ? tau_v[k + 1] : 0.0;
        y = ak;
        z = zk;
        givens(y, z, &c, &s);
        rot_cols(u, rows, k, k + 1, c, s);
        const double ak1 = ak * c - zk * s;
        bk1 = bk * c - ap * s;
        const double zk1 = bp * -s;
        ap1 = bk * s + ap * c;
        bp1 = bp * c;
        tau_u[k] = ak1;
        ak = ak1;
        bk = bk1;
        zk = zk1;
        ap = ap1;
        bp = bp1;
        aq = (k < cols - 2) ? tau_u[k + 2] : 0.0;
        y = bk;
        z = zk;
    }
    tau_v[cols - 2] = bk;
    tau_u[cols - 1] = ap;
}

// returns false when the sweep bound was reached
template <int R = 8>
__host__ __device__ inline bool diagonalise(double (*u)[3], double (*v)[3], double* tau_u, double* tau_v, int rows) {
    chop(tau_u, tau_v, 3);
    int b = 2;
    int guard = 0;
    while (b > 0) {
        if (++guard > QR_SWEEP_LIMIT) return false;
        if (tau_v[b - 1] == 0.0) {
            b -= 1;
        } else {
            int a = b - 1;
            while (a > 0 && tau_v[a - 1] != 0.0) a -= 1;
            const int n = b - a + 1;
            double u1[R][3], v1[3][3];
            for (int i = 0; i < rows; ++i) u1[i][0] = u1[i][1] = u1[i][2] = 0.0;
            for (int i = 0; i < 3; ++i) v1[i][0] = v1[i][1] = v1[i][2] = 0.0;
            for (int j = a; j <= b; ++j) {
                for (int i = 0; i < rows; ++i) u1[i][j - a] = u[i][j];
                for (int i = 0; i < 3; ++i) v1[i][j - a] = v[i][j];
            }
            qr_step(u1, v1, tau_u + a, tau_v + a, rows, n);
            for (int j = a; j <= b; ++j) {
                for (int i = 0; i < rows; ++i) u[i][j] = u1[i][j - a];
                for (int i = 0; i < 3; ++i) v[i][j] = v1[i][j - a];
            }
            chop(tau_u + a, tau_v + a, n);
        }
    }
    return true;
}

__host__ __device__ inline void singularise(double (*u)[3], double (*v)[3], double* d, int rows) {
    for (int j = 0; j < 3; ++j) {
        if (d[j] < 0.0) {
            for (int i = 0; i < 3; ++i) v[i][j] = -v[i][j];
            d[j] = -d[j];
        }
    }
    for (int i = 0; i < 3; ++i) {
        double d_max = d[i];
        int i_max = i;
        for (int j = i + 1; j < 3; ++j)
            if (d[j] > d_max) {
                d_max = d[j];
                i_max = j;
            }
        if (i_max != i) {
            double t = d[i];
            d[i] = d[i_max];
            d[i_max] = t;
            for (int y = 0; y < rows; ++y) {
                t = u[y][i];
                u[y][i] = u[y][i_max];
                u[y][i_max] = t;
            }
            for (int y = 0; y < 3; ++y) {
                t = v[y][i];
                v[y][i] = v[y][i_max];
                v[y][i_max] = t;
            }
        }
    }
}

// MinimiseQEF::place_feature_with_tangents; *ok = false if the QR bound hit
__host__ __device__ inline F3 minimise_qef(const Planes& t, bool* ok) {
    *ok = true;
    if (t.feature == PLANAR) return t.com;
    double u[8][3], v[3][3], d[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < 8; ++i) {
        u[i][0] = (double)t.normal[i].x;
        u[i][1] = (double)t.normal[i].y;
        u[i][2] = (double)t.normal[i].z;
    }
    double tau_v[2] = {0.0, 0.0};
    bidiagonalise(u, d, tau_v, 8);
    unpack(u, v, d, tau_v, 8);
    *ok = diagonalise(u, v, d, tau_v, 8);
    singularise(u, v, d, 8);
    if (t.feature == EDGE) {
        double s_min = 1.7976931348623157e308;
        int id = 0;
        for (int i = 0; i < 3; ++i)
            if (d[i] < s_min) {
                s_min = d[i];
                id = i;
            }
        d[id] = 0.0;
    }
    if (d[2] < 0.1) d[2] = 0.0;
    if (d[1] < 0.1) d[1] = 0.0;
    if (d[0] < 0.1) d[0] = 0.0;
    double w[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < 8; ++i) {
        const double b = (double)t.d[i];
        if (b != 0.0)
            for (int j = 0; j < 3; ++j) w[j] += b * u[i][j];
    }
    for (int i = 0; i < 3; ++i)
        if (d[i] != 0.0) w[i] /= d[i];
    double x[3];
    for (int i = 0; i < 3; ++i) {
        double s = 0.0;
        for (int j = 0; j < 3; ++j) s += w[j] * v[i][j];
        x[i] = s;
    }
    return add(t.com, f3((float)x[0], (float)x[1], (float)x[2]));
}

}  // namespace qef
}  // namespace iso
