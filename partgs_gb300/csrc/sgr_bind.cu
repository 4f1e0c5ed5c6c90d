// Superquadric -> surfel binding with a hand-written adjoint.
//
// Forward restates BlockGaussianModel.prepare_scaling_rot / update_alpha /
// get_verts / get_opacity (games/block_mesh_splatting/scene/
// block_gaussian_model.py:107-109, 178-256) with parametric_sq
// (games/block_mesh_splatting/utils/superquadric.py:10-14), signed_pow
// (games/block_mesh_splatting/utils/pytorch.py:28-29),
// quaternion_to_rotation_matrix (superquadric.py:93-107) and
// rot_to_quat_batch (utils/general_utils.py:34-87).
//
// Work layout: the frame (normal, tangents, scales, quaternion) is a
// per-triangle quantity, so one thread handles one triangle and loops over
// its N surfels; the backward scatters triangle-vertex gradients into a
// per-vertex buffer, and one CTA per superquadric reduces its vertices'
// contributions without atomics.
#include <cuda.h>
#include <cuda_runtime.h>

#include <climits>
#include <mutex>
#include <string>

#include "../../include/sgr.h"

namespace sgr {
void count_launches(int n);                      // sgr_api.cu
void set_last_error(const std::string& message); // sgr_api.cu
}  // namespace sgr

namespace sgrbind {

constexpr float kEps = 1e-8f;

struct F3 {
  float x, y, z;
};
__device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ F3 operator*(float s, F3 a) { return f3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ F3 operator/(F3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 cross(F3 a, F3 b) {
  return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float norm(F3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ float sigmoid(float x) { return 1.f / (1.f + expf(-x)); }
__device__ __forceinline__ float signed_pow(float t, float e) {
  const float s = t > 0.f ? 1.f : (t < 0.f ? -1.f : 0.f);
  return s * powf(fabsf(t), e);
}

// Per-superquadric transform: exponents, scale, rotation (row-major, w-first
// quaternion after F.normalize), translation.
struct SQ {
  float e1, e2;
  F3 S, t;
  float R[3][3];
  float q[4];      // normalised quaternion
  float rnorm;     // |sq_r| (clamped as F.normalize does)
};

__device__ __forceinline__ SQ load_sq(const sgr_bind_args& a, int b) {
  SQ s;
  s.e1 = sigmoid(a.sq_eps[2 * b]) * 1.8f + 0.1f;
  s.e2 = sigmoid(a.sq_eps[2 * b + 1]) * 1.8f + 0.1f;
  s.S = f3(expf(a.sq_s[3 * b]) + a.scale_block_min, expf(a.sq_s[3 * b + 1]) + a.scale_block_min,
           expf(a.sq_s[3 * b + 2]) + a.scale_block_min);
  s.t = f3(a.sq_t[3 * b], a.sq_t[3 * b + 1], a.sq_t[3 * b + 2]);
  const float r0 = a.sq_r[4 * b], r1 = a.sq_r[4 * b + 1], r2 = a.sq_r[4 * b + 2], r3 = a.sq_r[4 * b + 3];
  s.rnorm = fmaxf(sqrtf(r0 * r0 + r1 * r1 + r2 * r2 + r3 * r3), 1e-12f);
  const float w = r0 / s.rnorm, x = r1 / s.rnorm, y = r2 / s.rnorm, z = r3 / s.rnorm;
  s.q[0] = w; s.q[1] = x; s.q[2] = y; s.q[3] = z;
  s.R[0][0] = 1 - 2 * y * y - 2 * z * z; s.R[0][1] = 2 * x * y - 2 * z * w; s.R[0][2] = 2 * x * z + 2 * y * w;
  s.R[1][0] = 2 * x * y + 2 * z * w; s.R[1][1] = 1 - 2 * x * x - 2 * z * z; s.R[1][2] = 2 * y * z - 2 * x * w;
  s.R[2][0] = 2 * x * z - 2 * y * w; s.R[2][1] = 2 * y * z + 2 * x * w; s.R[2][2] = 1 - 2 * x * x - 2 * y * y;
  return s;
}

// Unit-superquadric point (times ratio) and the transformed vertex.
__device__ __forceinline__ F3 sq_point(float eta, float omega, float e1, float e2, float ratio) {
  const float ce = signed_pow(cosf(eta), e1), se = signed_pow(sinf(eta), e1);
  const float co = signed_pow(cosf(omega), e2), so = signed_pow(sinf(omega), e2);
  return f3(ce * so * ratio, se * ratio, ce * co * ratio);
}
__device__ __forceinline__ F3 sq_vertex(const SQ& s, F3 v) {
  const F3 w = f3(v.x * s.S.x, v.y * s.S.y, v.z * s.S.z);
  return f3(w.x * s.R[0][0] + w.y * s.R[1][0] + w.z * s.R[2][0] + s.t.x,
            w.x * s.R[0][1] + w.y * s.R[1][1] + w.z * s.R[2][1] + s.t.y,
            w.x * s.R[0][2] + w.y * s.R[1][2] + w.z * s.R[2][2] + s.t.z);
}

// Triangle frame and the quaternion of the (v1, v2, v0) column basis.
struct Frame {
  F3 t[3], e1, e2, nrm, v0, m, v1r, v1, v2i, v2u, v2;
  float n0, nv1, n1, n2u, s1, s2;
  float mat[3][3];
  float xq[4], qa[4];
  int ibest;
  float den, sign;
  float row[4];
  float quat[4];
};

__device__ void frame_forward(Frame& fr) {
  fr.e1 = fr.t[1] - fr.t[0];
  fr.e2 = fr.t[2] - fr.t[0];
  fr.nrm = cross(fr.e1, fr.e2);
  fr.n0 = norm(fr.nrm);
  fr.v0 = fr.nrm / (fr.n0 + kEps);
  fr.m = (fr.t[0] + fr.t[1] + fr.t[2]) / 3.f;
  fr.v1r = fr.t[1] - fr.m;
  fr.nv1 = norm(fr.v1r);
  fr.n1 = fr.nv1 + kEps;
  fr.v1 = fr.v1r / fr.n1;
  fr.v2i = fr.t[2] - fr.m;
  fr.v2u = fr.v2i - dot(fr.v2i, fr.v0) * fr.v0 - dot(fr.v2i, fr.v1) * fr.v1;
  fr.n2u = norm(fr.v2u);
  fr.v2 = fr.v2u / (fr.n2u + kEps);
  fr.s1 = fr.n1 / 2.f;
  fr.s2 = dot(fr.v2i, fr.v2) / 2.f;
  // matrix with columns v1, v2, v0 (row-major m[i][j])
  const F3 cols[3] = {fr.v1, fr.v2, fr.v0};
  for (int j = 0; j < 3; ++j) {
    fr.mat[0][j] = cols[j].x;
    fr.mat[1][j] = cols[j].y;
    fr.mat[2][j] = cols[j].z;
  }
  const float(&m)[3][3] = fr.mat;
  fr.xq[0] = 1.f + m[0][0] + m[1][1] + m[2][2];
  fr.xq[1] = 1.f + m[0][0] - m[1][1] - m[2][2];
  fr.xq[2] = 1.f - m[0][0] + m[1][1] - m[2][2];
  fr.xq[3] = 1.f - m[0][0] - m[1][1] + m[2][2];
  fr.ibest = 0;
  for (int k = 0; k < 4; ++k) {
    fr.qa[k] = fr.xq[k] > 0.f ? sqrtf(fr.xq[k]) : 0.f;
    if (fr.qa[k] > fr.qa[fr.ibest]) fr.ibest = k;
  }
  const int i = fr.ibest;
  const float qa2 = fr.qa[i] * fr.qa[i];
  if (i == 0) {
    fr.row[0] = qa2; fr.row[1] = m[2][1] - m[1][2]; fr.row[2] = m[0][2] - m[2][0]; fr.row[3] = m[1][0] - m[0][1];
  } else if (i == 1) {
    fr.row[0] = m[2][1] - m[1][2]; fr.row[1] = qa2; fr.row[2] = m[1][0] + m[0][1]; fr.row[3] = m[0][2] + m[2][0];
  } else if (i == 2) {
    fr.row[0] = m[0][2] - m[2][0]; fr.row[1] = m[1][0] + m[0][1]; fr.row[2] = qa2; fr.row[3] = m[1][2] + m[2][1];
  } else {
    fr.row[0] = m[1][0] - m[0][1]; fr.row[1] = m[2][0] + m[0][2]; fr.row[2] = m[2][1] + m[1][2]; fr.row[3] = qa2;
  }
  fr.den = 2.f * fmaxf(fr.qa[i], 0.1f);
  float out[4];
  for (int k = 0; k < 4; ++k) out[k] = fr.row[k] / fr.den;
  fr.sign = out[0] < 0.f ? -1.f : 1.f;
  for (int k = 0; k < 4; ++k) fr.quat[k] = fr.sign * out[k];
}

__device__ __forceinline__ void load_triangle(const sgr_bind_args& a, const SQ& s, int b, int f, Frame& fr, int vid[3]) {
  for (int k = 0; k < 3; ++k) {
    vid[k] = a.faces[((size_t)b * a.F + f) * 3 + k];
    const float eta = a.eta[(size_t)b * a.V + vid[k]];
    const float om = a.omega[(size_t)b * a.V + vid[k]];
    fr.t[k] = sq_vertex(s, sq_point(eta, om, s.e1, s.e2, a.ratio_block_scene));
  }
}

__device__ __forceinline__ void barycentric(const float* raw, float w[3]) {
  const float a0 = fmaxf(raw[0], 0.f) + 1e-8f, a1 = fmaxf(raw[1], 0.f) + 1e-8f, a2 = fmaxf(raw[2], 0.f) + 1e-8f;
  const float sum = a0 + a1 + a2;
  w[0] = a0 / sum;
  w[1] = a1 / sum;
  w[2] = a2 / sum;
}

__global__ void k_bind_forward(const sgr_bind_args a, float* __restrict__ xyz, float* __restrict__ log_scaling,
                               float* __restrict__ rotation, float* __restrict__ opacity) {
  const int fi = blockIdx.x * blockDim.x + threadIdx.x;
  if (fi >= a.B * a.F) return;
  const int b = fi / a.F, f = fi - b * a.F;
  const SQ s = load_sq(a, b);
  Frame fr;
  int vid[3];
  load_triangle(a, s, b, f, fr, vid);
  frame_forward(fr);
  const float op = sigmoid(a.sq_occ[b]);
  for (int n = 0; n < a.N; ++n) {
    const size_t si = (size_t)fi * a.N + n;
    float w[3];
    barycentric(a.alpha + si * 3, w);
    if (xyz) {
      const F3 p = w[0] * fr.t[0] + w[1] * fr.t[1] + w[2] * fr.t[2];
      xyz[3 * si] = p.x;
      xyz[3 * si + 1] = p.y;
      xyz[3 * si + 2] = p.z;
    }
    if (log_scaling) {
      const float sc = a.scale[(size_t)b * a.F * a.N + (size_t)f * a.N + n];
      log_scaling[2 * si] = logf(fmaxf(sc * fr.s1, 0.f) + kEps);
      log_scaling[2 * si + 1] = logf(fmaxf(sc * fr.s2, 0.f) + kEps);
    }
    if (rotation)
      for (int k = 0; k < 4; ++k) rotation[4 * si + k] = fr.quat[k];
    if (opacity) opacity[si] = op;
  }
}

// d(v / (|v| + eps)) given dy, v, |v|.
__device__ __forceinline__ F3 dnormalize(F3 dy, F3 v, float nv) {
  const float den = nv + kEps;
  F3 r = dy / den;
  if (nv > 0.f) r = r - (dot(dy, v) / (den * den * nv)) * v;
  return r;
}

__global__ void k_bind_backward_faces(const sgr_bind_args a, const float* __restrict__ d_xyz,
                                      const float* __restrict__ d_log, const float* __restrict__ d_rot,
                                      const float* __restrict__ d_op, float* __restrict__ dvert,
                                      float* __restrict__ dop_face) {
  const int fi = blockIdx.x * blockDim.x + threadIdx.x;
  if (fi >= a.B * a.F) return;
  const int b = fi / a.F, f = fi - b * a.F;
  const SQ s = load_sq(a, b);
  Frame fr;
  int vid[3];
  load_triangle(a, s, b, f, fr, vid);
  frame_forward(fr);
  F3 dt[3] = {f3(0, 0, 0), f3(0, 0, 0), f3(0, 0, 0)};
  float ds1 = 0.f, ds2 = 0.f, dq[4] = {0.f, 0.f, 0.f, 0.f}, dop = 0.f;
  for (int n = 0; n < a.N; ++n) {
    const size_t si = (size_t)fi * a.N + n;
    if (d_xyz) {
      float w[3];
      barycentric(a.alpha + si * 3, w);
      const F3 g = f3(d_xyz[3 * si], d_xyz[3 * si + 1], d_xyz[3 * si + 2]);
      for (int k = 0; k < 3; ++k) dt[k] = dt[k] + w[k] * g;
    }
    if (d_log) {
      const float sc = a.scale[(size_t)b * a.F * a.N + (size_t)f * a.N + n];
      const float x1 = sc * fr.s1, x2 = sc * fr.s2;
      if (x1 > 0.f) ds1 += d_log[2 * si] / (x1 + kEps) * sc;
      if (x2 > 0.f) ds2 += d_log[2 * si + 1] / (x2 + kEps) * sc;
    }
    if (d_rot)
      for (int k = 0; k < 4; ++k) dq[k] += d_rot[4 * si + k];
    if (d_op) dop += d_op[si];
  }
  dop_face[fi] = dop;

  // rot_to_quat_batch adjoint (only the selected candidate row carries gradient)
  float dm[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  {
    const int i = fr.ibest;
    float drow[4], dden = 0.f;
    for (int k = 0; k < 4; ++k) {
      const float dout = fr.sign * dq[k];
      drow[k] = dout / fr.den;
      dden -= dout * fr.row[k] / (fr.den * fr.den);
    }
    float dqa = (fr.qa[i] > 0.1f ? 2.f * dden : 0.f) + drow[i] * 2.f * fr.qa[i];
    const float dx = fr.xq[i] > 0.f ? dqa / (2.f * fr.qa[i]) : 0.f;
    // x_i in terms of the diagonal
    const float sgn[4][3] = {{1, 1, 1}, {1, -1, -1}, {-1, 1, -1}, {-1, -1, 1}};
    dm[0][0] += sgn[i][0] * dx;
    dm[1][1] += sgn[i][1] * dx;
    dm[2][2] += sgn[i][2] * dx;
    // off-diagonal entries of the selected row
    if (i == 0) {
      dm[2][1] += drow[1]; dm[1][2] -= drow[1];
      dm[0][2] += drow[2]; dm[2][0] -= drow[2];
      dm[1][0] += drow[3]; dm[0][1] -= drow[3];
    } else if (i == 1) {
      dm[2][1] += drow[0]; dm[1][2] -= drow[0];
      dm[1][0] += drow[2]; dm[0][1] += drow[2];
      dm[0][2] += drow[3]; dm[2][0] += drow[3];
    } else if (i == 2) {
      dm[0][2] += drow[0]; dm[2][0] -= drow[0];
      dm[1][0] += drow[1]; dm[0][1] += drow[1];
      dm[1][2] += drow[3]; dm[2][1] += drow[3];
    } else {
      dm[1][0] += drow[0]; dm[0][1] -= drow[0];
      dm[2][0] += drow[1]; dm[0][2] += drow[1];
      dm[2][1] += drow[2]; dm[1][2] += drow[2];
    }
  }
  // columns of the matrix are v1, v2, v0
  F3 dv1 = f3(dm[0][0], dm[1][0], dm[2][0]);
  F3 dv2 = f3(dm[0][1], dm[1][1], dm[2][1]);
  F3 dv0 = f3(dm[0][2], dm[1][2], dm[2][2]);
  float dn1 = ds1 / 2.f;
  F3 dv2i = (ds2 / 2.f) * fr.v2;
  dv2 = dv2 + (ds2 / 2.f) * fr.v2i;
  // v2 = v2u / (|v2u| + eps); v2u = v2i - <v2i,v0> v0 - <v2i,v1> v1
  const F3 dv2u = dnormalize(dv2, fr.v2u, fr.n2u);
  const float c0 = dot(fr.v2i, fr.v0), c1 = dot(fr.v2i, fr.v1);
  dv2i = dv2i + dv2u - dot(fr.v0, dv2u) * fr.v0 - dot(fr.v1, dv2u) * fr.v1;
  dv0 = dv0 - (c0 * dv2u + dot(fr.v0, dv2u) * fr.v2i);
  dv1 = dv1 - (c1 * dv2u + dot(fr.v1, dv2u) * fr.v2i);
  // v1 = v1r / n1, n1 = |v1r| + eps
  const float nv1 = fr.nv1;
  F3 dv1r = dv1 / fr.n1;
  if (nv1 > 0.f) dv1r = dv1r + ((dn1 - dot(dv1, fr.v1r) / (fr.n1 * fr.n1)) / nv1) * fr.v1r;
  // v0 = nrm / (|nrm| + eps), nrm = e1 x e2
  const F3 dnrm = dnormalize(dv0, fr.nrm, fr.n0);
  const F3 de1 = cross(fr.e2, dnrm);
  const F3 de2 = cross(dnrm, fr.e1);
  dt[1] = dt[1] + de1 + dv1r;
  dt[2] = dt[2] + de2 + dv2i;
  dt[0] = dt[0] - (de1 + de2);
  const F3 dmean = (-1.f / 3.f) * (dv1r + dv2i);
  for (int k = 0; k < 3; ++k) {
    dt[k] = dt[k] + dmean;
    float* o = dvert + ((size_t)b * a.V + vid[k]) * 3;
    atomicAdd(o, dt[k].x);
    atomicAdd(o + 1, dt[k].y);
    atomicAdd(o + 2, dt[k].z);
  }
}

__device__ __forceinline__ float block_sum(float v, float* sh) {
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  float t = 0.f;
  for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
  return t;
}

// One CTA per superquadric: vertex gradients -> superquadric parameters.
__global__ void k_bind_backward_sq(const sgr_bind_args a, const float* __restrict__ dvert,
                                   const float* __restrict__ dop_face, float* __restrict__ d_sq_s,
                                   float* __restrict__ d_sq_r, float* __restrict__ d_sq_t,
                                   float* __restrict__ d_sq_eps, float* __restrict__ d_sq_occ) {
  __shared__ float sh[32];
  const int b = blockIdx.x;
  const SQ s = load_sq(a, b);
  // accumulators: de1, de2, dS(3), dR(9), dt(3), dop
  float acc[18];
  for (int k = 0; k < 18; ++k) acc[k] = 0.f;
  for (int vtx = threadIdx.x; vtx < a.V; vtx += blockDim.x) {
    const float* g = dvert + ((size_t)b * a.V + vtx) * 3;
    const F3 dvp = f3(g[0], g[1], g[2]);
    const float eta = a.eta[(size_t)b * a.V + vtx], om = a.omega[(size_t)b * a.V + vtx];
    const float cE = cosf(eta), sE = sinf(eta), cO = cosf(om), sO = sinf(om);
    const float ce = signed_pow(cE, s.e1), se = signed_pow(sE, s.e1);
    const float co = signed_pow(cO, s.e2), so = signed_pow(sO, s.e2);
    const float ratio = a.ratio_block_scene;
    const F3 v = f3(ce * so * ratio, se * ratio, ce * co * ratio);
    const F3 w = f3(v.x * s.S.x, v.y * s.S.y, v.z * s.S.z);
    acc[14] += dvp.x;
    acc[15] += dvp.y;
    acc[16] += dvp.z;
    const float wv[3] = {w.x, w.y, w.z};
    const float gv[3] = {dvp.x, dvp.y, dvp.z};
    float dw[3];
    for (int k = 0; k < 3; ++k) {
      dw[k] = s.R[k][0] * gv[0] + s.R[k][1] * gv[1] + s.R[k][2] * gv[2];
      for (int j = 0; j < 3; ++j) acc[5 + 3 * k + j] += wv[k] * gv[j];
    }
    acc[2] += dw[0] * v.x;
    acc[3] += dw[1] * v.y;
    acc[4] += dw[2] * v.z;
    const float dvx = dw[0] * s.S.x, dvy = dw[1] * s.S.y, dvz = dw[2] * s.S.z;
    const float dce = ratio * (dvx * so + dvz * co), dso = ratio * dvx * ce;
    const float dse = ratio * dvy, dco = ratio * dvz * ce;
    // d/de sign(t)|t|^e = sign(t)|t|^e ln|t| (zero at t = 0)
    auto dpow = [](float val, float base) { return base != 0.f ? val * logf(fabsf(base)) : 0.f; };
    acc[0] += dce * dpow(ce, cE) + dse * dpow(se, sE);
    acc[1] += dco * dpow(co, cO) + dso * dpow(so, sO);
  }
  for (int fi = threadIdx.x; fi < a.F; fi += blockDim.x) acc[17] += dop_face[(size_t)b * a.F + fi];
  float tot[18];
  for (int k = 0; k < 18; ++k) tot[k] = block_sum(acc[k], sh);
  if (threadIdx.x != 0) return;
  const float se1 = sigmoid(a.sq_eps[2 * b]), se2 = sigmoid(a.sq_eps[2 * b + 1]);
  d_sq_eps[2 * b] = tot[0] * 1.8f * se1 * (1.f - se1);
  d_sq_eps[2 * b + 1] = tot[1] * 1.8f * se2 * (1.f - se2);
  for (int k = 0; k < 3; ++k) d_sq_s[3 * b + k] = tot[2 + k] * expf(a.sq_s[3 * b + k]);
  for (int k = 0; k < 3; ++k) d_sq_t[3 * b + k] = tot[14 + k];
  const float so_ = sigmoid(a.sq_occ[b]);
  d_sq_occ[b] = tot[17] * so_ * (1.f - so_);
  // quaternion_to_rotation_matrix adjoint, then F.normalize
  float dR[3][3];
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < 3; ++j) dR[k][j] = tot[5 + 3 * k + j];
  const float w = s.q[0], x = s.q[1], y = s.q[2], z = s.q[3];
  float dq[4];
  dq[0] = -2 * z * dR[0][1] + 2 * y * dR[0][2] + 2 * z * dR[1][0] - 2 * x * dR[1][2] - 2 * y * dR[2][0] + 2 * x * dR[2][1];
  dq[1] = 2 * y * dR[0][1] + 2 * z * dR[0][2] + 2 * y * dR[1][0] - 4 * x * dR[1][1] - 2 * w * dR[1][2] + 2 * z * dR[2][0] +
          2 * w * dR[2][1] - 4 * x * dR[2][2];
  dq[2] = -4 * y * dR[0][0] + 2 * x * dR[0][1] + 2 * w * dR[0][2] + 2 * x * dR[1][0] + 2 * z * dR[1][2] - 2 * w * dR[2][0] +
          2 * z * dR[2][1] - 4 * y * dR[2][2];
  dq[3] = -4 * z * dR[0][0] - 2 * w * dR[0][1] + 2 * x * dR[0][2] + 2 * w * dR[1][0] - 4 * z * dR[1][1] + 2 * y * dR[1][2] +
          2 * x * dR[2][0] + 2 * y * dR[2][1];
  const float qd = w * dq[0] + x * dq[1] + y * dq[2] + z * dq[3];
  for (int k = 0; k < 4; ++k) d_sq_r[4 * b + k] = (dq[k] - s.q[k] * qd) / s.rnorm;
}

thread_local std::string g_bind_error;

int check_args(const sgr_bind_args* a) {
  if (!a || a->B < 0 || a->V < 0 || a->F < 0 || a->N < 0) return SGR_ERR_INVALID_ARGUMENT;
  // surfel, face and vertex indices are 32-bit in the kernels
  if ((long long)a->B * a->F * (a->N > 0 ? a->N : 1) > INT_MAX || (long long)a->B * a->V * 3 > INT_MAX) {
    sgr::set_last_error("superquadric binding: more than 2^31 - 1 surfels, faces or vertex coordinates");
    return SGR_ERR_UNSUPPORTED;
  }
  if (a->B > 0 && (!a->sq_s || !a->sq_r || !a->sq_t || !a->sq_eps || !a->sq_occ)) return SGR_ERR_INVALID_ARGUMENT;
  if ((size_t)a->B * a->F > 0 && (!a->eta || !a->omega || !a->faces || !a->alpha || !a->scale))
    return SGR_ERR_INVALID_ARGUMENT;
  return SGR_OK;
}

// ---------------------------------------------------------------------------
// Scratch of the allocation-free backward (sgr_bind_backward_static): one
// file-scope device array, so calling it allocates nothing.  Its bytes are
// per-vertex gradient sums and per-triangle opacity sums, accumulated with
// atomics, so each call clears the bytes it uses before its kernels run.
// ---------------------------------------------------------------------------
constexpr size_t kBindStaticScratchBytes = size_t(4) << 20;   // 4 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_bind_static_scratch[kBindStaticScratchBytes];

std::mutex g_static_mu;
void* g_static_ptr[kMaxDevices] = {};
unsigned long long g_static_ctx[kMaxDevices] = {};   // id of the context the address belongs to

// Id of the current device's current context, through the driver entry
// points the runtime hands out (so the library does not link libcuda).
int current_context_id(unsigned long long* id) {
  using get_current_fn = CUresult (*)(CUcontext*);
  using get_id_fn = CUresult (*)(CUcontext, unsigned long long*);
  static get_current_fn get_current = nullptr;
  static get_id_fn get_id = nullptr;
  if (!get_current || !get_id) {
    void* f0 = nullptr;
    void* f1 = nullptr;
    cudaDriverEntryPointQueryResult q0, q1;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess || !f0 || !f1) {
      sgr::set_last_error("sgr_bind_backward_static: the driver does not provide cuCtxGetCurrent / cuCtxGetId");
      return SGR_ERR_CUDA;
    }
    get_current = reinterpret_cast<get_current_fn>(f0);
    get_id = reinterpret_cast<get_id_fn>(f1);
  }
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, id) != CUDA_SUCCESS) {
    sgr::set_last_error("sgr_bind_backward_static: no current CUDA context");
    return SGR_ERR_CUDA;
  }
  return SGR_OK;
}

// Device address of the array on the current device, looked up with that
// device current: once per device, and again when the device's context has
// changed since (after cudaDeviceReset the module is loaded anew and the
// array may sit elsewhere).
int static_scratch(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    sgr::set_last_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    return SGR_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    sgr::set_last_error("sgr_bind_backward_static: device ordinal beyond the supported 64");
    return SGR_ERR_UNSUPPORTED;
  }
  // make the device's primary context current (initialised) before asking for it
  if ((e = cudaSetDevice(dev)) != cudaSuccess) {
    sgr::set_last_error(std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    return SGR_ERR_CUDA;
  }
  unsigned long long ctx = 0;
  int rc = current_context_id(&ctx);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(g_static_mu);
  if (!g_static_ptr[dev] || g_static_ctx[dev] != ctx) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_bind_static_scratch);
    if (e != cudaSuccess || !p) {
      sgr::set_last_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return SGR_ERR_CUDA;
    }
    g_static_ptr[dev] = p;
    g_static_ctx[dev] = ctx;
  }
  *out = g_static_ptr[dev];
  return SGR_OK;
}

}  // namespace sgrbind

using namespace sgrbind;

extern "C" {

int sgr_bind_forward(const sgr_bind_args* a, float* xyz, float* log_scaling, float* rotation, float* opacity,
                     void* stream) {
  int rc = check_args(a);
  if (rc) return rc;
  const int n = (int)((long long)a->B * a->F);   // at most INT_MAX (check_args)
  if (n == 0 || a->N == 0) return SGR_OK;
  k_bind_forward<<<(n + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(*a, xyz, log_scaling, rotation,
                                                                                  opacity);
  sgr::count_launches(1);
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

size_t sgr_bind_scratch_bytes(const sgr_bind_args* a) {
  if (!a) return 0;
  const size_t dv = ((size_t)a->B * a->V * 3 * 4 + 255) & ~(size_t)255;
  return dv + (size_t)a->B * a->F * 4;
}

int sgr_bind_backward(const sgr_bind_args* a, const float* d_xyz, const float* d_log_scaling, const float* d_rotation,
                      const float* d_opacity, float* d_sq_s, float* d_sq_r, float* d_sq_t, float* d_sq_eps,
                      float* d_sq_occ, void* scratch, void* stream) {
  int rc = check_args(a);
  if (rc) return rc;
  if (a->B == 0) return SGR_OK;
  if (!d_sq_s || !d_sq_r || !d_sq_t || !d_sq_eps || !d_sq_occ || !scratch) return SGR_ERR_INVALID_ARGUMENT;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  float* dvert = static_cast<float*>(scratch);
  const size_t dv = ((size_t)a->B * a->V * 3 * 4 + 255) & ~(size_t)255;
  float* dop_face = reinterpret_cast<float*>(static_cast<char*>(scratch) + dv);
  if (cudaMemsetAsync(scratch, 0, sgr_bind_scratch_bytes(a), st) != cudaSuccess) return SGR_ERR_CUDA;
  const int n = (int)((long long)a->B * a->F);   // at most INT_MAX (check_args)
  if (n > 0 && a->N > 0) {
    k_bind_backward_faces<<<(n + 127) / 128, 128, 0, st>>>(*a, d_xyz, d_log_scaling, d_rotation, d_opacity, dvert,
                                                            dop_face);
    sgr::count_launches(1);
  }
  k_bind_backward_sq<<<a->B, 256, 0, st>>>(*a, dvert, dop_face, d_sq_s, d_sq_r, d_sq_t, d_sq_eps, d_sq_occ);
  sgr::count_launches(1);
  return cudaGetLastError() == cudaSuccess ? SGR_OK : SGR_ERR_CUDA;
}

// sgr_bind_backward with its scratch in this library's fixed device array
// instead of a caller buffer; the same kernels, the same results.  For
// callers that cannot allocate device memory where they call the backward:
// a host that binds the C ABI without a device allocator of its own (it
// holds only the buffers it was handed), or a loop that must not enter
// cudaMalloc, which synchronises the device.
//   * Limit: sgr_bind_scratch_bytes(a) <= 4 MiB; larger shapes return
//     SGR_ERR_WORKSPACE and say so in sgr_last_error_message.
//   * One array per device: calls that overlap on a device (other streams,
//     other host threads) race on it; the caller serialises them.
//   * The first call on a device looks the array up (cudaGetSymbolAddress)
//     with that device current; make that first call before any stream
//     capture.
//   * The array must start each call at zero; the call clears the bytes it
//     uses with cudaMemsetAsync on `stream` before its kernels.
int sgr_bind_backward_static(const sgr_bind_args* a, const float* d_xyz, const float* d_log_scaling,
                             const float* d_rotation, const float* d_opacity, float* d_sq_s, float* d_sq_r,
                             float* d_sq_t, float* d_sq_eps, float* d_sq_occ, void* stream) {
  int rc = check_args(a);
  if (rc) return rc;
  if (a->B == 0) return SGR_OK;
  const size_t need = sgr_bind_scratch_bytes(a);
  if (need > kBindStaticScratchBytes) {
    sgr::set_last_error("sgr_bind_backward_static: the shape needs " + std::to_string(need) +
                        " bytes of scratch, above the fixed " + std::to_string(kBindStaticScratchBytes) +
                        "; use sgr_bind_backward with a caller buffer");
    return SGR_ERR_WORKSPACE;
  }
  void* scratch = nullptr;
  if ((rc = static_scratch(&scratch))) return rc;
  return sgr_bind_backward(a, d_xyz, d_log_scaling, d_rotation, d_opacity, d_sq_s, d_sq_r, d_sq_t, d_sq_eps,
                           d_sq_occ, scratch, stream);
}

}  // extern "C"
