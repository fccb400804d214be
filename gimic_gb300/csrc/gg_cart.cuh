// Value, gradient and Laplacian of the Cartesian component x^i y^j z^k f(r^2)
// (l = i + j + k <= 3) as straight-line code, one case per component:
//   phi = X f1, X = x^i y^j z^k;  d/dx phi = i x^(i-1) y^j z^k f1 - 2 x X f2;
//   lap = [i(i-1) x^(i-2) y^j z^k + (y, z alike)] f1 - 2 (2l + 3) X f2 + 4 r^2 X f3
// with f1 = sum c e^{-a r^2}, f2 = sum a c e^{-a r^2}, f3 = sum a^2 c e^{-a r^2}
// (src/libgimic/caos.f90:39-64 for the gradient).  cart_case_id() maps the
// packed exponents i | j << 4 | k << 8 to the case number.
#pragma once
#include <type_traits>

namespace gg {

// f(integral_constant<int, I>) for I = I0 .. N-1, unrolled at compile time
template <int I0, int N, typename F>
__device__ __forceinline__ void static_for(F&& f) {
  if constexpr (I0 < N) {
    f(std::integral_constant<int, I0>{});
    static_for<I0 + 1, N>(f);
  }
}

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

// Straight-line forms for a component known at compile time, in the order
// of cart_case_id (kCartStdCode[id] = i * 100 + j * 10 + k): used when a
// shell's functions are stored in that order (the component is then a
// compile-time function of its position in the shell).  Terms whose
// coefficient is zero are left out at compile time instead of multiplied.
constexpr int kCartStdCode[20] = {0, 100, 10, 1, 200, 110, 101, 20, 11, 2, 300, 210, 201, 120, 111, 102, 30, 21, 12, 3};
constexpr int kCartBase[4] = {0, 1, 4, 10};  // case id of a shell's first component, by l

template <int E>
__device__ __forceinline__ float cart_pw(float v, float v2) {
  static_assert(E >= 1 && E <= 3, "power");
  if constexpr (E == 1) return v;
  else if constexpr (E == 2) return v2;
  else return v2 * v;
}

// K x^A y^B z^C f
template <int K, int A, int B, int C>
__device__ __forceinline__ float cart_term(const CartPow& p, float f) {
  float m = f;
  if constexpr (A > 0) m = cart_pw<A>(p.x, p.x2) * m;
  if constexpr (B > 0) m = cart_pw<B>(p.y, p.y2) * m;
  if constexpr (C > 0) m = cart_pw<C>(p.z, p.z2) * m;
  if constexpr (K != 1) m = static_cast<float>(K) * m;
  return m;
}

// x^A y^B z^C (A + B + C > 0)
template <int A, int B, int C>
__device__ __forceinline__ float cart_mono(const CartPow& p) {
  static_assert(A + B + C > 0, "constant monomial");
  if constexpr (A > 0) {
    float m = cart_pw<A>(p.x, p.x2);
    if constexpr (B > 0) m = m * cart_pw<B>(p.y, p.y2);
    if constexpr (C > 0) m = m * cart_pw<C>(p.z, p.z2);
    return m;
  } else if constexpr (B > 0) {
    float m = cart_pw<B>(p.y, p.y2);
    if constexpr (C > 0) m = m * cart_pw<C>(p.z, p.z2);
    return m;
  } else {
    return cart_pw<C>(p.z, p.z2);
  }
}

// phi, grad phi and (kLap) the Laplacian of case ID from the shell's radial
// sums: f1, m2f2 = -2 f2 and lq = 4 r^2 f3 - 2 (2l + 3) f2 (the Laplacian's
// coefficient of the monomial).  Same quantities as cart_case.
template <int ID, bool kLap>
__device__ __forceinline__ void cart_std(const CartPow& p, float f1, float m2f2, float lq, float* phi, float* gx,
                                         float* gy, float* gz, float* lap) {
  constexpr int code = kCartStdCode[ID], A = code / 100, B = (code / 10) % 10, C = code % 10;
  float tX, xl;  // -2 f2 X and the Laplacian's X term
  if constexpr (A + B + C == 0) {
    *phi = f1;
    tX = m2f2;
    xl = lq;
  } else {
    const float X = cart_mono<A, B, C>(p);
    *phi = X * f1;
    tX = X * m2f2;
    xl = X * lq;
  }
  if constexpr (A > 0) *gx = fmaf(p.x, tX, cart_term<A, A - 1, B, C>(p, f1));
  else *gx = p.x * tX;
  if constexpr (B > 0) *gy = fmaf(p.y, tX, cart_term<B, A, B - 1, C>(p, f1));
  else *gy = p.y * tX;
  if constexpr (C > 0) *gz = fmaf(p.z, tX, cart_term<C, A, B, C - 1>(p, f1));
  else *gz = p.z * tX;
  if constexpr (kLap) {
    // l <= 3: at most one exponent reaches 2, so the second derivatives are one term
    if constexpr (A >= 2) *lap = cart_term<A * (A - 1), A - 2, B, C>(p, f1) + xl;
    else if constexpr (B >= 2) *lap = cart_term<B * (B - 1), A, B - 2, C>(p, f1) + xl;
    else if constexpr (C >= 2) *lap = cart_term<C * (C - 1), A, B, C - 2>(p, f1) + xl;
    else *lap = xl;
  }
}

}  // namespace gg
