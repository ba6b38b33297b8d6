// Forward-mode (tangent) arithmetic for the force- and stress-loss
// gradients.
//
// A Dual carries a value and its derivative along one direction of the
// atom positions and cell strains (v + eps t).  The plain FP32 path's
// kernels are templates over the scalar type: instantiated with float they
// are the plain path, instantiated with Dual they run the same operations
// on (value, tangent) pairs, so the weight-gradient reductions return both
// grad_theta E and its derivative along the direction -- the mixed second
// derivative a force or stress loss needs (the double backward of
// torch.autograd.grad(..., create_graph=True) followed by loss.backward()).
//
// The helpers below have a float overload that is exactly the plain path's
// expression, so the float instantiation compiles to the same code.
#pragma once
#include <type_traits>
#include "common.cuh"

namespace mlff {

struct Dual {
    float v, t;
};
struct Dual4 {
    Dual x, y, z, w;
};

template <class T> struct Vec4Of;
template <> struct Vec4Of<float> { using type = float4; };
template <> struct Vec4Of<Dual> { using type = Dual4; };
template <class T> using Vec4 = typename Vec4Of<T>::type;

template <class T> constexpr bool is_dual_v = std::is_same<T, Dual>::value;

// silu''(z) = s (1 - s) (2 + z (1 - 2 s)), s = sigmoid(z)
__device__ __forceinline__ float d2silu_f(float x) {
    const float s = sigmoid_f(x);
    return s * (1.0f - s) * (2.0f + x * (1.0f - 2.0f * s));
}

// ------------------------------------------------------------ operators
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.t + b.t}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.t - b.t}; }
__device__ __forceinline__ Dual operator+(Dual a, float b) { return {a.v + b, a.t}; }
__device__ __forceinline__ Dual operator+(float a, Dual b) { return {a + b.v, b.t}; }
__device__ __forceinline__ Dual operator-(Dual a, float b) { return {a.v - b, a.t}; }
__device__ __forceinline__ Dual operator-(float a, Dual b) { return {a - b.v, -b.t}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, fmaf(a.t, b.v, a.v * b.t)}; }
__device__ __forceinline__ Dual operator*(Dual a, float b) { return {a.v * b, a.t * b}; }
__device__ __forceinline__ Dual operator*(float a, Dual b) { return {a * b.v, a * b.t}; }
__device__ __forceinline__ Dual operator/(Dual a, float b) { return {a.v / b, a.t / b}; }
__device__ __forceinline__ Dual operator/(float a, Dual b) {
    const float q = a / b.v;
    return {q, -q * b.t / b.v};
}
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
    const float q = a.v / b.v;
    return {q, (a.t - q * b.t) / b.v};
}
__device__ __forceinline__ Dual& operator+=(Dual& a, Dual b) { return a = a + b; }

// ------------------------------------------------------------- helpers
template <class T> __device__ __forceinline__ T tzero() { return T{}; }
template <class T> __device__ __forceinline__ T tone();
template <> __device__ __forceinline__ float tone<float>() { return 1.0f; }
template <> __device__ __forceinline__ Dual tone<Dual>() { return {1.0f, 0.0f}; }

// value v with tangent t (the tangent is dropped for float)
template <class T> __device__ __forceinline__ T tmake(float v, float t);
template <> __device__ __forceinline__ float tmake<float>(float v, float) { return v; }
template <> __device__ __forceinline__ Dual tmake<Dual>(float v, float t) { return {v, t}; }

__device__ __forceinline__ float tval(float a) { return a; }
__device__ __forceinline__ float tval(Dual a) { return a.v; }

__device__ __forceinline__ float tfma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ Dual tfma(Dual a, float b, Dual c) { return {fmaf(a.v, b, c.v), fmaf(a.t, b, c.t)}; }
__device__ __forceinline__ Dual tfma(float a, Dual b, Dual c) { return {fmaf(a, b.v, c.v), fmaf(a, b.t, c.t)}; }
__device__ __forceinline__ Dual tfma(Dual a, Dual b, Dual c) {
    return {fmaf(a.v, b.v, c.v), fmaf(a.t, b.v, fmaf(a.v, b.t, c.t))};
}

__device__ __forceinline__ float texp(float a) { return expf(a); }
__device__ __forceinline__ Dual texp(Dual a) {
    const float e = expf(a.v);
    return {e, e * a.t};
}
__device__ __forceinline__ float tcos(float a) { return cosf(a); }
__device__ __forceinline__ Dual tcos(Dual a) { return {cosf(a.v), -sinf(a.v) * a.t}; }
__device__ __forceinline__ float tsin(float a) { return sinf(a); }
__device__ __forceinline__ Dual tsin(Dual a) { return {sinf(a.v), cosf(a.v) * a.t}; }

__device__ __forceinline__ float tsilu(float z) { return silu_f(z); }
__device__ __forceinline__ Dual tsilu(Dual z) { return {silu_f(z.v), dsilu_f(z.v) * z.t}; }
__device__ __forceinline__ float tdsilu(float z) { return dsilu_f(z); }
__device__ __forceinline__ Dual tdsilu(Dual z) { return {dsilu_f(z.v), d2silu_f(z.v) * z.t}; }

// |(x, y, z)| rounded as pair_distance; the tangent is 0 at the origin
// (torch.norm's subgradient there)
__device__ __forceinline__ float tdist(float x, float y, float z) { return pair_distance(x, y, z); }
__device__ __forceinline__ Dual tdist(Dual x, Dual y, Dual z) {
    const float d = pair_distance(x.v, y.v, z.v);
    const float t = d > 0.0f ? (x.v * x.t + y.v * y.t + z.v * z.t) / d : 0.0f;
    return {d, t};
}

__device__ __forceinline__ float4 tvec4(float x, float y, float z, float w) { return make_float4(x, y, z, w); }
__device__ __forceinline__ Dual4 tvec4(Dual x, Dual y, Dual z, Dual w) { return {x, y, z, w}; }

__device__ __forceinline__ void tatomic_add(float* p, float v) { atomicAdd(p, v); }
__device__ __forceinline__ void tatomic_add(Dual* p, Dual v) {
    atomicAdd(&p->v, v.v);
    atomicAdd(&p->t, v.t);
}

}  // namespace mlff
