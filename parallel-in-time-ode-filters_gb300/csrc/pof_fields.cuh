// Built-in vector fields (value and Jacobian) for on-device EK1
// linearization.  The fields are those of pof/ivp.py:7-152 plus the
// (a, b, c) FitzHugh-Nagumo form used by the benchmark configurations.
#pragma once

#include "pof_linalg.cuh"

namespace pof {

enum FieldId : int {
  FIELD_USER = 0,           // (H, c) supplied by the caller
  FIELD_LOGISTIC = 1,       // p = (r):             y' = r y (1 - y)                 pof/ivp.py:7-14
  FIELD_LOTKAVOLTERRA = 2,  // p = (a, b, c, d)                                      pof/ivp.py:17-31
  FIELD_VANDERPOL = 3,      // p = (mu)                                              pof/ivp.py:34-41
  FIELD_FITZHUGHNAGUMO = 4, // p = (a, b, 1/tau, I)                                  pof/ivp.py:44-60
  FIELD_FHN_CLASSIC = 5,    // p = (a, b, c): c (y1 - y1^3/3 + y2), -(y1 - a + b y2)/c
  FIELD_ROBER = 6,          // p = (k1, k2, k3)                                      pof/ivp.py:63-79
  FIELD_RIGID_BODY = 7,     // p = (p0, p1, p2)                                      pof/ivp.py:82-90
  FIELD_SEIR = 8,           // p = (p0, p1, p2, p3)                                  pof/ivp.py:93-108
  FIELD_THREEBODY = 9,      // p = (mu)                                              pof/ivp.py:111-126
  FIELD_HENONHEILES = 10,   // p = (p)                                               pof/ivp.py:137-152
  FIELD_FHN_RD = 11,        // p = (a, b, c, kv, kw): FitzHugh-Nagumo on a periodic 1-D grid of d / 2
                            // cells (method of lines), y = (v_0..v_{m-1}, w_0..w_{m-1}); any even d;
                            // linearized by the dense path's kernel
  FIELD_COUNT = 12,
};

__host__ __device__ inline int field_dim(int id) {
  switch (id) {
    case FIELD_LOGISTIC: return 1;
    case FIELD_LOTKAVOLTERRA:
    case FIELD_VANDERPOL:
    case FIELD_FITZHUGHNAGUMO:
    case FIELD_FHN_CLASSIC: return 2;
    case FIELD_ROBER:
    case FIELD_RIGID_BODY: return 3;
    case FIELD_SEIR:
    case FIELD_THREEBODY:
    case FIELD_HENONHEILES: return 4;
    case FIELD_FHN_RD: return 0;  // any even d
    default: return -1;
  }
}

__host__ __device__ inline int field_nparams(int id) {
  switch (id) {
    case FIELD_LOGISTIC:
    case FIELD_VANDERPOL:
    case FIELD_THREEBODY:
    case FIELD_HENONHEILES: return 1;
    case FIELD_FHN_CLASSIC:
    case FIELD_ROBER:
    case FIELD_RIGID_BODY: return 3;
    case FIELD_LOTKAVOLTERRA:
    case FIELD_FITZHUGHNAGUMO:
    case FIELD_SEIR: return 4;
    case FIELD_FHN_RD: return 5;
    default: return 0;
  }
}

// f(y) and J = df/dy (row-major DY x DY) of field `id` with parameters p.
template <typename T, int DY>
__device__ __forceinline__ void field_eval(int id, const T* __restrict__ p, const T* __restrict__ y, T* f, T* J) {
#pragma unroll
  for (int i = 0; i < DY * DY; ++i) J[i] = T(0);
  if constexpr (DY == 1) {
    if (id == FIELD_LOGISTIC) {
      const T r = p[0];
      f[0] = r * y[0] * (T(1) - y[0]);
      J[0] = r * (T(1) - T(2) * y[0]);
    }
  } else if constexpr (DY == 2) {
    if (id == FIELD_LOTKAVOLTERRA) {
      const T a = p[0], b = p[1], c = p[2], d = p[3];
      f[0] = a * y[0] - b * y[0] * y[1];
      f[1] = -c * y[1] + d * y[0] * y[1];
      J[0] = a - b * y[1];
      J[1] = -b * y[0];
      J[2] = d * y[1];
      J[3] = -c + d * y[0];
    } else if (id == FIELD_VANDERPOL) {
      const T mu = p[0];
      f[0] = y[1];
      f[1] = mu * ((T(1) - y[0] * y[0]) * y[1] - y[0]);
      J[1] = T(1);
      J[2] = mu * (T(-2) * y[0] * y[1] - T(1));
      J[3] = mu * (T(1) - y[0] * y[0]);
    } else if (id == FIELD_FITZHUGHNAGUMO) {
      const T a = p[0], b = p[1], tinv = p[2], l = p[3];
      const T v = y[0], w = y[1];
      f[0] = v - (v * v * v) / T(3) - w + l;
      f[1] = tinv * (v + a - b * w);
      J[0] = T(1) - v * v;
      J[1] = T(-1);
      J[2] = tinv;
      J[3] = -tinv * b;
    } else if (id == FIELD_FHN_CLASSIC) {
      const T a = p[0], b = p[1], c = p[2];
      const T v = y[0], w = y[1];
      f[0] = c * (v - v * v * v / T(3) + w);
      f[1] = -(v - a + b * w) / c;
      J[0] = c * (T(1) - v * v);
      J[1] = c;
      J[2] = T(-1) / c;
      J[3] = -b / c;
    }
  } else if constexpr (DY == 3) {
    if (id == FIELD_ROBER) {
      const T k1 = p[0], k2 = p[1], k3 = p[2];
      f[0] = -k1 * y[0] + k3 * y[1] * y[2];
      f[1] = k1 * y[0] - k2 * y[1] * y[1] - k3 * y[1] * y[2];
      f[2] = k2 * y[1] * y[1];
      J[0] = -k1; J[1] = k3 * y[2]; J[2] = k3 * y[1];
      J[3] = k1; J[4] = T(-2) * k2 * y[1] - k3 * y[2]; J[5] = -k3 * y[1];
      J[6] = T(0); J[7] = T(2) * k2 * y[1]; J[8] = T(0);
    } else if (id == FIELD_RIGID_BODY) {
      f[0] = p[0] * y[1] * y[2];
      f[1] = p[1] * y[0] * y[2];
      f[2] = p[2] * y[0] * y[1];
      J[1] = p[0] * y[2]; J[2] = p[0] * y[1];
      J[3] = p[1] * y[2]; J[5] = p[1] * y[0];
      J[6] = p[2] * y[1]; J[7] = p[2] * y[0];
    }
  } else if constexpr (DY == 4) {
    if (id == FIELD_SEIR) {
      const T s = p[1] / p[3];
      f[0] = -s * y[0] * y[2];
      f[1] = s * y[0] * y[2] - p[0] * y[1];
      f[2] = p[0] * y[1] - p[2] * y[2];
      f[3] = p[2] * y[2];
      J[0] = -s * y[2]; J[2] = -s * y[0];
      J[4] = s * y[2]; J[5] = -p[0]; J[6] = s * y[0];
      J[9] = p[0]; J[10] = -p[2];
      J[14] = p[2];
    } else if (id == FIELD_HENONHEILES) {
      const T q = p[0];
      f[0] = y[2];
      f[1] = y[3];
      f[2] = -y[0] - T(2) * q * y[0] * y[1];
      f[3] = -y[1] - q * (y[0] * y[0] - y[1] * y[1]);
      J[2] = T(1);
      J[7] = T(1);
      J[8] = T(-1) - T(2) * q * y[1]; J[9] = T(-2) * q * y[0];
      J[12] = T(-2) * q * y[0]; J[13] = T(-1) + T(2) * q * y[1];
    } else if (id == FIELD_THREEBODY) {
      const T mu = p[0], mp = T(1) - p[0];
      const T ax = y[0] + mu, bx = y[0] - mp, yy = y[1];
      const T r1s = ax * ax + yy * yy, r2s = bx * bx + yy * yy;
      const T r1 = sqrt(r1s), r2 = sqrt(r2s);
      const T D1 = r1s * r1, D2 = r2s * r2;          // |.|^3
      const T D1b = D1 * r1s, D2b = D2 * r2s;        // |.|^5
      f[0] = y[2];
      f[1] = y[3];
      f[2] = y[0] + T(2) * y[3] - mp * ax / D1 - mu * bx / D2;
      f[3] = y[1] - T(2) * y[2] - mp * yy / D1 - mu * yy / D2;
      J[2] = T(1);
      J[7] = T(1);
      J[8] = T(1) - mp * (T(1) / D1 - T(3) * ax * ax / D1b) - mu * (T(1) / D2 - T(3) * bx * bx / D2b);
      J[9] = mp * T(3) * ax * yy / D1b + mu * T(3) * bx * yy / D2b;
      J[11] = T(2);
      J[12] = mp * T(3) * ax * yy / D1b + mu * T(3) * bx * yy / D2b;
      J[13] = T(1) - mp * (T(1) / D1 - T(3) * yy * yy / D1b) - mu * (T(1) / D2 - T(3) * yy * yy / D2b);
      J[14] = T(-2);
    }
  }
}

}  // namespace pof
