// Value, gradient and Laplacian of the Cartesian component x^i y^j z^k f(r^2)
// (l = i + j + k <= 3) as straight-line code, one case per component:
//   phi = X f1, X = x^i y^j z^k;  d/dx phi = i x^(i-1) y^j z^k f1 - 2 x X f2;
//   lap = [i(i-1) x^(i-2) y^j z^k + (y, z alike)] f1 - 2 (2l + 3) X f2 + 4 r^2 X f3
// with f1 = sum c e^{-a r^2}, f2 = sum a c e^{-a r^2}, f3 = sum a^2 c e^{-a r^2}
// (src/libgimic/caos.f90:39-64 for the gradient).  cart_case_id() maps the
// packed exponents i | j << 4 | k << 8 to the case number.
#pragma once

namespace gg {

struct CartPow {
  float x, y, z, x2, y2, z2;
};

__device__ __forceinline__ CartPow cart_pow(float x, float y, float z) {
  CartPow p;
  p.x = x;
  p.y = y;
  p.z = z;
  p.x2 = x * x;
  p.y2 = y * y;
  p.z2 = z * z;
  return p;
}

inline int cart_case_id(int packed) {
  const int i = packed & 15, j = (packed >> 4) & 15, k = (packed >> 8) & 15;
  if (i == 0 && j == 0 && k == 0) return 0;
  if (i == 1 && j == 0 && k == 0) return 1;
  if (i == 0 && j == 1 && k == 0) return 2;
  if (i == 0 && j == 0 && k == 1) return 3;
  if (i == 2 && j == 0 && k == 0) return 4;
  if (i == 1 && j == 1 && k == 0) return 5;
  if (i == 1 && j == 0 && k == 1) return 6;
  if (i == 0 && j == 2 && k == 0) return 7;
  if (i == 0 && j == 1 && k == 1) return 8;
  if (i == 0 && j == 0 && k == 2) return 9;
  if (i == 3 && j == 0 && k == 0) return 10;
  if (i == 2 && j == 1 && k == 0) return 11;
  if (i == 2 && j == 0 && k == 1) return 12;
  if (i == 1 && j == 2 && k == 0) return 13;
  if (i == 1 && j == 1 && k == 1) return 14;
  if (i == 1 && j == 0 && k == 2) return 15;
  if (i == 0 && j == 3 && k == 0) return 16;
  if (i == 0 && j == 2 && k == 1) return 17;
  if (i == 0 && j == 1 && k == 2) return 18;
  if (i == 0 && j == 0 && k == 3) return 19;
  return -1;
}

__device__ __forceinline__ void cart_case(int id, const CartPow& p, float f1, float f2, float f3, float* phi,
                                          float* gx, float* gy, float* gz, float* lap) {
  const float x = p.x, y = p.y, z = p.z, x2 = p.x2, y2 = p.y2, z2 = p.z2;
  float X, dx, dy, dz, sec;  // X, d/dx of the monomial, ..., sum of its second derivatives
  switch (id) {
    case 0:  // x^0 y^0 z^0
      X = 1.f;
      dx = 0.f;
      dy = 0.f;
      dz = 0.f;
      sec = 0.f;
      break;
    case 1:  // x^1 y^0 z^0
      X = x;
      dx = 1.f;
      dy = 0.f;
      dz = 0.f;
      sec = 0.f;
      break;
    case 2:  // x^0 y^1 z^0
      X = y;
      dx = 0.f;
      dy = 1.f;
      dz = 0.f;
      sec = 0.f;
      break;
    case 3:  // x^0 y^0 z^1
      X = z;
      dx = 0.f;
      dy = 0.f;
      dz = 1.f;
      sec = 0.f;
      break;
    case 4:  // x^2 y^0 z^0
      X = x2;
      dx = 2.f * x;
      dy = 0.f;
      dz = 0.f;
      sec = 2.f * 1.f;
      break;
    case 5:  // x^1 y^1 z^0
      X = x * y;
      dx = y;
      dy = x;
      dz = 0.f;
      sec = 0.f;
      break;
    case 6:  // x^1 y^0 z^1
      X = x * z;
      dx = z;
      dy = 0.f;
      dz = x;
      sec = 0.f;
      break;
    case 7:  // x^0 y^2 z^0
      X = y2;
      dx = 0.f;
      dy = 2.f * y;
      dz = 0.f;
      sec = 2.f * 1.f;
      break;
    case 8:  // x^0 y^1 z^1
      X = y * z;
      dx = 0.f;
      dy = z;
      dz = y;
      sec = 0.f;
      break;
    case 9:  // x^0 y^0 z^2
      X = z2;
      dx = 0.f;
      dy = 0.f;
      dz = 2.f * z;
      sec = 2.f * 1.f;
      break;
    case 10:  // x^3 y^0 z^0
      X = x2 * x;
      dx = 3.f * x2;
      dy = 0.f;
      dz = 0.f;
      sec = 6.f * x;
      break;
    case 11:  // x^2 y^1 z^0
      X = x2 * y;
      dx = 2.f * x * y;
      dy = x2;
      dz = 0.f;
      sec = 2.f * y;
      break;
    case 12:  // x^2 y^0 z^1
      X = x2 * z;
      dx = 2.f * x * z;
      dy = 0.f;
      dz = x2;
      sec = 2.f * z;
      break;
    case 13:  // x^1 y^2 z^0
      X = x * y2;
      dx = y2;
      dy = 2.f * x * y;
      dz = 0.f;
      sec = 2.f * x;
      break;
    case 14:  // x^1 y^1 z^1
      X = x * y * z;
      dx = y * z;
      dy = x * z;
      dz = x * y;
      sec = 0.f;
      break;
    case 15:  // x^1 y^0 z^2
      X = x * z2;
      dx = z2;
      dy = 0.f;
      dz = 2.f * x * z;
      sec = 2.f * x;
      break;
    case 16:  // x^0 y^3 z^0
      X = y2 * y;
      dx = 0.f;
      dy = 3.f * y2;
      dz = 0.f;
      sec = 6.f * y;
      break;
    case 17:  // x^0 y^2 z^1
      X = y2 * z;
      dx = 0.f;
      dy = 2.f * y * z;
      dz = y2;
      sec = 2.f * z;
      break;
    case 18:  // x^0 y^1 z^2
      X = y * z2;
      dx = 0.f;
      dy = z2;
      dz = 2.f * y * z;
      sec = 2.f * y;
      break;
    case 19:  // x^0 y^0 z^3
      X = z2 * z;
      dx = 0.f;
      dy = 0.f;
      dz = 3.f * z2;
      sec = 6.f * z;
      break;
    default:
      X = dx = dy = dz = sec = 0.f;
  }
  const float lsum = static_cast<float>(2 * (2 * (id == 0 ? 0 : id < 4 ? 1 : id < 10 ? 2 : 3) + 3));
  *phi = X * f1;
  *gx = fmaf(dx, f1, -2.f * x * X * f2);
  *gy = fmaf(dy, f1, -2.f * y * X * f2);
  *gz = fmaf(dz, f1, -2.f * z * X * f2);
  if (lap) *lap = fmaf(sec, f1, X * fmaf(4.f * (x2 + y2 + z2), f3, -lsum * f2));
}

}  // namespace gg
