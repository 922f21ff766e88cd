// nt2cuda/expr.cuh -- device mirror of an NT2 table expression and its
// compile-time lowering into one fused elementwise kernel.
//
// An NT2 assignment `out = f(g(X), Y, s)` is a Boost.Proto tree whose leaves
// are table terminals and splatted scalars
// (modules/core/sdk/include/nt2/core/container/dsl/expression.hpp:161-191);
// NT2 evaluates it per index in the SIMD transform loop
// (modules/core/base/include/nt2/core/functions/simd/transform.hpp:40-57),
// recursing through the tree (modules/core/sdk/include/nt2/dsl/functions/generic/run.hpp:180-222)
// down to terminal loads and scalar splats
// (modules/core/sdk/include/nt2/dsl/functions/container/terminal.hpp:77-129,180-198).
//
// Here the same tree is a plain C++ type: term<T> (a table in HBM),
// scal<T> (a scalar), node<Tag, Children...>.  `regs<E,V>` mirrors the tree
// with V register lanes per terminal; `load` fills them with 16-byte loads,
// `get(l)` evaluates the tree on lane l.  `assign<T,E>` pairs an output table
// with an expression, and a program is a list of assigns (several for NT2's
// tie(), modules/core/container/table/include/nt2/core/functions/expr/tie.hpp:40-74).
// k_transform<Prog> is the single fused kernel for the whole statement.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <limits>
#include <type_traits>
#include "math.cuh"
#include "bs_x2.cuh"
#include "trig.cuh"
#include "memory.cuh"

namespace nt2cuda {

// ------------------------------------------------------------------- tags
// Functor tags, named after NT2's (boost::simd::tag::plus_, nt2::tag::exp_, ...).
namespace tag {
struct plus_ {}; struct minus_ {}; struct multiplies_ {}; struct divides_ {};
struct unary_minus_ {}; struct fma_ {}; struct fnms_ {}; struct sqr_ {}; struct sqrt_ {};
struct rec_ {}; struct abs_ {}; struct exp_ {}; struct log_ {}; struct erfc_ {};
struct exp2_ {}; struct exp10_ {}; struct log2_ {}; struct log10_ {}; struct expm1_ {}; struct log1p_ {};
struct normcdf_ {}; struct fastnormcdf_ {}; struct max_ {}; struct min_ {};
struct adds_ {}; struct subs_ {}; struct selinc_ {}; struct seldec_ {}; struct if_else_ {};
struct if_zero_else_one_ {}; struct is_less_ {}; struct is_greater_ {};
struct is_less_equal_ {}; struct is_greater_equal_ {}; struct is_equal_ {};
struct is_not_equal_ {}; struct oneminus_ {}; struct minusone_ {}; struct cast_ {};
// cast<uint8_t> of a float the statement keeps in [0, 256) (see trunc_u8 below)
struct trunc_u8_ {};
// trigonometric functors, reduced element by element as NT2's scalar code does;
// simd128_<T> evaluates T over 16-byte packs as NT2's 128-bit SIMD code does
// (see regs<node<simd128_<...>>> below)
struct sin_ {}; struct cos_ {}; struct tan_ {}; struct sinpi_ {}; struct cospi_ {};
struct cot_ {}; struct tanpi_ {}; struct cotpi_ {}; struct sind_ {}; struct cosd_ {}; struct tand_ {}; struct cotd_ {};
template <class T> struct simd128_ {};
struct asin_ {}; struct acos_ {}; struct atan_ {}; struct atan2_ {};
struct sinh_ {}; struct cosh_ {}; struct tanh_ {};
struct pow_ {};
// the rest of NT2's exponential family (expx2s_ is the two-argument expx2)
struct cbrt_ {}; struct sqrt1pm1_ {}; struct exprecneg_ {}; struct exprecnegc_ {}; struct expx2_ {};
struct atanh_ {}; struct acosh_ {}; struct asinh_ {}; struct hypot_ {}; struct coth_ {}; struct sinhc_ {};
struct expx2s_ {}; struct pow_abs_ {}; struct logspace_add_ {}; struct logspace_sub_ {};
// steps of the composed trigonometric functors (csc = rec(sin), asind = indeg(asin), ...)
struct indeg_ {}; struct inrad_ {}; struct invpi_mul_ {}; struct oneo_180_mul_ {}; struct pio2_minus_ {};
struct cscpi_nan_ {}; struct secpi_nan_ {}; struct nan_if_zero_ {}; struct sinc_fix_ {};
struct atan2d_ {}; struct nbd_atan2_ {}; struct proper_tanpi_ {};
// fast_sin ... fast_cotd: K 0 sin, 1 cos, 2 tan, 3 cot; U 0 radian, 1 pi, 2 degree
template <int K, int U> struct fast_ {};
}  // namespace tag

// ------------------------------------------------------------ tree nodes
template <class T> struct term { const T* p; };
template <class T> struct scal { T v; };
template <class Tag, class... C> struct node;
template <class Tag, class A> struct node<Tag, A> { A a; };
template <class Tag, class A, class B> struct node<Tag, A, B> { A a; B b; };
template <class Tag, class A, class B, class C> struct node<Tag, A, B, C> { A a; B b; C c; };

template <class T, class E> struct assign { T* out; E e; };

// ---------------------------------------------------------------- functors
// One lane of each functor.  F selects fused multiply-adds (see math.cuh).
template <class Tag, bool F> struct fn;

#define NT2CUDA_BIN(TAG, EXPR)                                                   \
  template <bool F> struct fn<tag::TAG, F> {                                     \
    template <class A, class B>                                                  \
    __device__ __forceinline__ static auto apply(A a, B b) { return EXPR; }      \
  };
#define NT2CUDA_UN(TAG, EXPR)                                                    \
  template <bool F> struct fn<tag::TAG, F> {                                     \
    template <class A>                                                           \
    __device__ __forceinline__ static auto apply(A a) { return EXPR; }           \
  };

namespace detail {
template <class T> __device__ __forceinline__ T add(T a, T b) {
  if constexpr (std::is_floating_point<T>::value) return math::add(a, b); else return (T)(a + b); }
template <class T> __device__ __forceinline__ T sub(T a, T b) {
  if constexpr (std::is_floating_point<T>::value) return math::sub(a, b); else return (T)(a - b); }
template <class T> __device__ __forceinline__ T mul(T a, T b) {
  if constexpr (std::is_floating_point<T>::value) return math::mul(a, b); else return (T)(a * b); }
template <class T> __device__ __forceinline__ T dv(T a, T b) {
  if constexpr (std::is_floating_point<T>::value) return math::div(a, b); else return (T)(a / b); }
template <bool F, class T> __device__ __forceinline__ T madd(T a, T b, T c) {
  if constexpr (std::is_floating_point<T>::value) return math::madd<F>(a, b, c); else return (T)(a * b + c); }
template <bool F, class T> __device__ __forceinline__ T nmsub(T a, T b, T c) {
  if constexpr (std::is_floating_point<T>::value) return math::nmsub<F>(a, b, c); else return (T)(c - a * b); }
// saturated add/sub of unsigned integers (boost/simd/arithmetic/functions/scalar/adds.hpp:65)
template <class T> __device__ __forceinline__ T adds(T a, T b) {
  if constexpr (std::is_floating_point<T>::value) return math::add(a, b);
  else if constexpr (std::is_unsigned<T>::value) { T s = (T)(a + b); return s < a ? (T)~T(0) : s; }
  else {
    using W = long long; W s = (W)a + (W)b;
    W lo = (W)std::numeric_limits<T>::min(), hi = (W)std::numeric_limits<T>::max();
    return (T)(s < lo ? lo : (s > hi ? hi : s));
  }
}
template <class T> __device__ __forceinline__ T subs(T a, T b) {
  if constexpr (std::is_floating_point<T>::value) return math::sub(a, b);
  else if constexpr (std::is_unsigned<T>::value) { return a > b ? (T)(a - b) : (T)0; }
  else {
    using W = long long; W s = (W)a - (W)b;
    W lo = (W)std::numeric_limits<T>::min(), hi = (W)std::numeric_limits<T>::max();
    return (T)(s < lo ? lo : (s > hi ? hi : s));
  }
}
}  // namespace detail

NT2CUDA_BIN(plus_, detail::add(a, (A)b))
NT2CUDA_BIN(minus_, detail::sub(a, (A)b))
NT2CUDA_BIN(multiplies_, detail::mul(a, (A)b))
NT2CUDA_BIN(divides_, detail::dv(a, (A)b))
NT2CUDA_BIN(max_, (a > (A)b ? a : (A)b))
NT2CUDA_BIN(min_, (a < (A)b ? a : (A)b))
NT2CUDA_BIN(adds_, detail::adds(a, (A)b))
NT2CUDA_BIN(subs_, detail::subs(a, (A)b))
NT2CUDA_BIN(is_less_, (bool)(a < b))
NT2CUDA_BIN(is_greater_, (bool)(a > b))
NT2CUDA_BIN(is_less_equal_, (bool)(a <= b))
NT2CUDA_BIN(is_greater_equal_, (bool)(a >= b))
NT2CUDA_BIN(is_equal_, (bool)(a == b))
NT2CUDA_BIN(is_not_equal_, (bool)(a != b))
// selinc(c,x) = c ? x+1 : x ; seldec(c,x) = c ? x-1 : x
// (boost/simd/boolean/functions/scalar/selinc.hpp:27, seldec.hpp:27)
NT2CUDA_BIN(selinc_, (a ? (B)(b + 1) : b))
NT2CUDA_BIN(seldec_, (a ? (B)(b - 1) : b))
NT2CUDA_BIN(atan2_, trig::atan2<F>(a, (A)b))
NT2CUDA_BIN(pow_, math::pow<F>(a, (A)b))
NT2CUDA_BIN(pow_abs_, math::pow_abs<F>(a, (A)b))
NT2CUDA_BIN(logspace_add_, math::logspace_add<F>(a, (A)b))
NT2CUDA_BIN(logspace_sub_, math::logspace_sub<F>(a, (A)b))
NT2CUDA_BIN(expx2s_, math::expx2<F>(a, (A)b))
NT2CUDA_UN(cbrt_, math::cbrt<F>(a))
NT2CUDA_UN(indeg_, trig::indeg(a))
NT2CUDA_UN(inrad_, trig::inrad(a))
NT2CUDA_UN(invpi_mul_, trig::invpi_mul(a))
NT2CUDA_UN(oneo_180_mul_, trig::oneo_180_mul(a))
NT2CUDA_UN(pio2_minus_, trig::pio2_minus(a))
NT2CUDA_BIN(cscpi_nan_, trig::cscpi_nan(a, (A)b))
NT2CUDA_BIN(secpi_nan_, trig::secpi_nan(a, (A)b))
NT2CUDA_UN(nan_if_zero_, (a == (A)0 ? (A)NAN : a))
NT2CUDA_BIN(sinc_fix_, trig::sinc_fix(a, (A)b))
NT2CUDA_BIN(atan2d_, trig::indeg(trig::atan2<F>(a, (A)b)))
NT2CUDA_BIN(nbd_atan2_, trig::nbd_atan2<F>(a, (A)b))
NT2CUDA_UN(proper_tanpi_, trig::proper_tanpi<F>(a))
template <int K, int U, bool F> struct fn<tag::fast_<K, U>, F> {
  template <class A> __device__ __forceinline__ static auto apply(A a) { return trig::fast<K, U, F>(a); }
};
NT2CUDA_UN(sqrt1pm1_, math::sqrt1pm1<F>(a))
NT2CUDA_UN(exprecneg_, math::exprecneg<F>(a))
NT2CUDA_UN(exprecnegc_, math::exprecnegc<F>(a))
NT2CUDA_UN(expx2_, math::expx2<F>(a))
NT2CUDA_UN(atanh_, math::atanh<F>(a))
NT2CUDA_UN(acosh_, math::acosh<F>(a))
NT2CUDA_UN(asinh_, math::asinh<F>(a))
NT2CUDA_UN(coth_, math::coth<F>(a))
NT2CUDA_UN(sinhc_, math::sinhc<F>(a))
NT2CUDA_BIN(hypot_, math::hypot(a, (A)b))
NT2CUDA_UN(unary_minus_, (A)(-a))
NT2CUDA_UN(sqr_, detail::mul(a, a))
NT2CUDA_UN(sqrt_, math::sqrt_(a))
NT2CUDA_UN(rec_, detail::dv((A)1, a))
NT2CUDA_UN(abs_, (a < (A)0 ? (A)(-a) : a))
NT2CUDA_UN(oneminus_, detail::sub((A)1, a))
NT2CUDA_UN(minusone_, detail::sub(a, (A)1))
NT2CUDA_UN(exp_, math::exp<F>(a))
NT2CUDA_UN(log_, math::log<F>(a))
NT2CUDA_UN(exp2_, math::exp2<F>(a))
NT2CUDA_UN(exp10_, math::exp10<F>(a))
NT2CUDA_UN(log2_, math::log2<F>(a))
NT2CUDA_UN(log10_, math::log10<F>(a))
NT2CUDA_UN(expm1_, math::expm1<F>(a))
NT2CUDA_UN(log1p_, math::log1p<F>(a))
NT2CUDA_UN(erfc_, math::erfc<F>(a))
NT2CUDA_UN(normcdf_, math::normcdf<F>(a))
NT2CUDA_UN(fastnormcdf_, math::fastnormcdf<F>(a))
NT2CUDA_UN(sinh_, math::sinh<F>(a))
NT2CUDA_UN(cosh_, math::cosh<F>(a))
NT2CUDA_UN(tanh_, math::tanh<F>(a))
NT2CUDA_UN(asin_, trig::asin<F>(a))
NT2CUDA_UN(acos_, trig::acos<F>(a))
NT2CUDA_UN(atan_, trig::atan<F>(a))
// trunc_u8(y) = cast<uint8_t>(y) for a float y in [0, 256), where the cast truncates toward
// zero: 2^23 + y rounded toward zero is 2^23 + floor(y), whose low byte is the result.
// Used where the statement bounds y (rgb2grey's weights sum below 1); a full-rate add in
// place of the quarter-rate float-to-integer conversion.
NT2CUDA_UN(trunc_u8_, (uint8_t)(__float_as_uint(__fadd_rz((float)a, 8388608.0f)) & 0xFFu))
// if_zero_else_one(c) = c ? 0 : 1 (boost/simd/boolean/functions/scalar/if_zero_else_one.hpp:28-50);
// the result type is the caller's element type, carried by the node.
#undef NT2CUDA_BIN
#undef NT2CUDA_UN

template <bool F> struct fn<tag::fma_, F> {
  template <class A, class B, class C>
  __device__ __forceinline__ static A apply(A a, B b, C c) { return detail::madd<F>(a, (A)b, (A)c); }
};
template <bool F> struct fn<tag::fnms_, F> {
  template <class A, class B, class C>
  __device__ __forceinline__ static A apply(A a, B b, C c) { return detail::nmsub<F>(a, (A)b, (A)c); }
};
template <bool F> struct fn<tag::if_else_, F> {
  template <class A, class B, class C>
  __device__ __forceinline__ static B apply(A a, B b, C c) { return a ? b : (B)c; }
};

// ------------------------------------------------------------ value types
template <class E> struct value_of;
template <class T> struct value_of<term<T>> { using type = T; };
template <class T> struct value_of<scal<T>> { using type = T; };
// Result type of a functor from its argument types (spelled out rather than
// deduced from fn::apply, which is device code): comparisons give bool,
// selinc/seldec/if_else give their second argument's type, everything else
// its first argument's type.
template <class Tag, class... A> struct tag_result;
template <class Tag, class A, class... R> struct tag_result<Tag, A, R...> { using type = A; };
#define NT2CUDA_BOOL_RESULT(TAG) \
  template <class A, class B> struct tag_result<tag::TAG, A, B> { using type = bool; };
NT2CUDA_BOOL_RESULT(is_less_)
NT2CUDA_BOOL_RESULT(is_greater_)
NT2CUDA_BOOL_RESULT(is_less_equal_)
NT2CUDA_BOOL_RESULT(is_greater_equal_)
NT2CUDA_BOOL_RESULT(is_equal_)
NT2CUDA_BOOL_RESULT(is_not_equal_)
#undef NT2CUDA_BOOL_RESULT
template <class A, class B> struct tag_result<tag::selinc_, A, B> { using type = B; };
template <class A, class B> struct tag_result<tag::seldec_, A, B> { using type = B; };
template <class A, class B, class C> struct tag_result<tag::if_else_, A, B, C> { using type = B; };

template <class Tag, class... C> struct value_of<node<Tag, C...>> {
  using type = typename tag_result<Tag, typename value_of<C>::type...>::type;
};
// if_zero_else_one and cast carry their result type in a scal<R> second child that is never read.
template <class A, class R> struct value_of<node<tag::if_zero_else_one_, A, scal<R>>> { using type = R; };
template <class A, class R> struct value_of<node<tag::cast_, A, scal<R>>> { using type = R; };
template <class A> struct tag_result<tag::trunc_u8_, A> { using type = uint8_t; };

// nt2::cast<R>(x) (nt2/operator/functions/container/cast.hpp:133-150): integer -> floating goes
// through tofloat, floating -> unsigned through touint then narrowing groups, floating -> signed
// through toint; each of those is a plain C conversion of the scalar
// (boost/simd/arithmetic/functions/scalar/touint.hpp:31-36, swar/functions/scalar/group.hpp:20-27).
// Defined for values the target type (or its 32-bit widening) represents, as in NT2.
template <class R, class A> __device__ __forceinline__ R cast_value(A a)
{
  if constexpr (std::is_same<R, float>::value && std::is_unsigned<A>::value && sizeof(A) < 4) {
    // exact: 2^23 + a is a float whose low mantissa bits are a; subtracting 2^23 leaves a.
    // An integer add and a float add instead of the quarter-rate integer-to-float conversion.
    return __fsub_rn(__uint_as_float(0x4B000000u | (uint32_t)a), 8388608.0f);
  } else if constexpr (std::is_floating_point<A>::value && std::is_integral<R>::value && sizeof(R) < 4) {
    if constexpr (std::is_unsigned<R>::value) return (R)(uint32_t)a; else return (R)(int32_t)a;
  } else {
    return (R)a;
  }
}

// Smallest element size among the terminals (drives the lane count).
template <class E> struct min_elem;
template <class T> struct min_elem<term<T>> { static constexpr int value = (int)sizeof(T); };
template <class T> struct min_elem<scal<T>> { static constexpr int value = 1 << 20; };
constexpr int min_of() { return 1 << 20; }
template <class... R> constexpr int min_of(int a, R... r) { return a < min_of(r...) ? a : min_of(r...); }
template <class Tag, class... C> struct min_elem<node<Tag, C...>> {
  static constexpr int value = min_of(min_elem<C>::value...);
};

// ---------------------------------------------------------- register lanes
template <class E, int V> struct regs;

template <class T, int V> struct regs<term<T>, V> {
  T v[V];
  template <bool Stream> __device__ __forceinline__ void load(const term<T>& t, size_t i) {
    mem::load_vec<T, V, Stream>(t.p, i, v);
  }
  template <bool Stream> __device__ __forceinline__ void load_one(const term<T>& t, size_t i, int l) {
    v[l] = t.p[i];
  }
  template <bool F> __device__ __forceinline__ T get(const term<T>&, int l) const { return v[l]; }
};

template <class T, int V> struct regs<scal<T>, V> {
  template <bool Stream> __device__ __forceinline__ void load(const scal<T>&, size_t) {}
  template <bool Stream> __device__ __forceinline__ void load_one(const scal<T>&, size_t, int) {}
  template <bool F> __device__ __forceinline__ T get(const scal<T>& s, int) const { return s.v; }
};

// FP32 exp, log, erfc, normcdf, fastnormcdf and cbrt nodes run two lanes per packed instruction
// (nt2cuda/bs_x2.cuh, bit-identical to the one-lane functors over every
// float): asked for an even lane, the node computes that lane and the next
// one and hands the latter out when it is asked for (the kernels ask for
// lanes 0..V-1 in order, as the trigonometric nodes below also rely on).
template <class Tag> struct x2_unary { static constexpr bool value = false; };
template <> struct x2_unary<tag::exp_> { static constexpr bool value = true; };
template <> struct x2_unary<tag::log_> { static constexpr bool value = true; };
template <> struct x2_unary<tag::fastnormcdf_> { static constexpr bool value = true; };
template <> struct x2_unary<tag::erfc_> { static constexpr bool value = true; };
template <> struct x2_unary<tag::normcdf_> { static constexpr bool value = true; };
template <> struct x2_unary<tag::cbrt_> { static constexpr bool value = true; };
template <class Tag, bool F> __device__ __forceinline__ float2 x2_apply(float2 a)
{
  float2 pos, neg;
  if constexpr (std::is_same<Tag, tag::exp_>::value) {
    return x2::exp<F>(a);
  } else if constexpr (std::is_same<Tag, tag::cbrt_>::value) {
    return x2::cbrt<F>(a);
  } else if constexpr (std::is_same<Tag, tag::log_>::value) {
    return x2::log<F>(a);
  } else if constexpr (std::is_same<Tag, tag::erfc_>::value) {   // math::erfc
    const float2 r1 = x2::erfc_abs<F>(make_float2(fabsf(a.x), fabsf(a.y)));
    const float2 two_m = x2::sub(x2::splat(2.0f), r1);
    return make_float2((a.x < 0.0f) ? two_m.x : r1.x, (a.y < 0.0f) ? two_m.y : r1.y);
  } else if constexpr (std::is_same<Tag, tag::normcdf_>::value) {   // math::normcdf, as normcdf_pair's first
    x2::normcdf_pair<F>(a, pos, neg);
    return pos;
  } else {
    x2::fastnormcdf_pair<F>(a, pos, neg);
    return pos;
  }
}

template <class Tag, class A, int V> struct regs<node<Tag, A>, V> {
  static constexpr bool kPair = x2_unary<Tag>::value && V % 2 == 0 &&
                                std::is_same<typename value_of<A>::type, float>::value;
  regs<A, V> ra;
  mutable float pend;   // the odd lane of the last pair (kPair)
  template <bool S> __device__ __forceinline__ void load(const node<Tag, A>& n, size_t i) { ra.template load<S>(n.a, i); }
  template <bool S> __device__ __forceinline__ void load_one(const node<Tag, A>& n, size_t i, int l) { ra.template load_one<S>(n.a, i, l); }
  template <bool F> __device__ __forceinline__ auto get(const node<Tag, A>& n, int l) const {
    if constexpr (kPair) {
      if (l & 1) return pend;
      const float a0 = ra.template get<F>(n.a, l);       // lane l before lane l + 1: the
      const float a1 = ra.template get<F>(n.a, l + 1);   // operand may be a paired node too
      const float2 r = x2_apply<Tag, F>(make_float2(a0, a1));
      pend = r.y;
      return r.x;
    } else {
      return fn<Tag, F>::apply(ra.template get<F>(n.a, l));
    }
  }
};

// FP32 pow and pow_abs nodes run two lanes per packed instruction as above
// (x2::pow, x2::pow_abs: bit-identical to math::pow, math::pow_abs).
template <class Tag> struct x2_binary { static constexpr bool value = false; };
template <> struct x2_binary<tag::pow_> { static constexpr bool value = true; };
template <> struct x2_binary<tag::pow_abs_> { static constexpr bool value = true; };

template <class Tag, class A, class B, int V> struct regs<node<Tag, A, B>, V> {
  static constexpr bool kPair = x2_binary<Tag>::value && V % 2 == 0 &&
                                std::is_same<typename value_of<A>::type, float>::value &&
                                std::is_same<typename value_of<B>::type, float>::value;
  regs<A, V> ra; regs<B, V> rb;
  mutable float pend;   // the odd lane of the last pair (kPair)
  template <bool S> __device__ __forceinline__ void load(const node<Tag, A, B>& n, size_t i) {
    ra.template load<S>(n.a, i); rb.template load<S>(n.b, i);
  }
  template <bool S> __device__ __forceinline__ void load_one(const node<Tag, A, B>& n, size_t i, int l) {
    ra.template load_one<S>(n.a, i, l); rb.template load_one<S>(n.b, i, l);
  }
  template <bool F> __device__ __forceinline__ auto get(const node<Tag, A, B>& n, int l) const {
    if constexpr (std::is_same<Tag, tag::if_zero_else_one_>::value) {
      using R = typename value_of<node<Tag, A, B>>::type;
      return ra.template get<F>(n.a, l) ? R(0) : R(1);
    } else if constexpr (std::is_same<Tag, tag::cast_>::value) {
      using R = typename value_of<node<Tag, A, B>>::type;
      return cast_value<R>(ra.template get<F>(n.a, l));
    } else if constexpr (kPair) {
      if (l & 1) return pend;
      const float a0 = ra.template get<F>(n.a, l), a1 = ra.template get<F>(n.a, l + 1);
      const float b0 = rb.template get<F>(n.b, l), b1 = rb.template get<F>(n.b, l + 1);
      const float2 r = std::is_same<Tag, tag::pow_>::value ? x2::pow<F>(make_float2(a0, a1), make_float2(b0, b1))
                                                           : x2::pow_abs<F>(make_float2(a0, a1), make_float2(b0, b1));
      pend = r.y;
      return r.x;
    } else {
      return fn<Tag, F>::apply(ra.template get<F>(n.a, l), rb.template get<F>(n.b, l));
    }
  }
};

template <class Tag, class A, class B, class C, int V> struct regs<node<Tag, A, B, C>, V> {
  regs<A, V> ra; regs<B, V> rb; regs<C, V> rc;
  template <bool S> __device__ __forceinline__ void load(const node<Tag, A, B, C>& n, size_t i) {
    ra.template load<S>(n.a, i); rb.template load<S>(n.b, i); rc.template load<S>(n.c, i);
  }
  template <bool S> __device__ __forceinline__ void load_one(const node<Tag, A, B, C>& n, size_t i, int l) {
    ra.template load_one<S>(n.a, i, l); rb.template load_one<S>(n.b, i, l); rc.template load_one<S>(n.c, i, l);
  }
  template <bool F> __device__ __forceinline__ auto get(const node<Tag, A, B, C>& n, int l) const {
    return fn<Tag, F>::apply(ra.template get<F>(n.a, l), rb.template get<F>(n.b, l), rc.template get<F>(n.c, l));
  }
};

// Trigonometric nodes.  NT2's SIMD code reduces the arguments of a whole pack
// with one method chosen from the pack's largest |x| (nt2cuda/trig.cuh), so in
// the simd128_ form a lane's value depends on its neighbours; the plain tags
// are NT2's scalar code, each element on its own.  Either way the node
// computes all lanes of a group when asked for the group's first lane and
// hands out the rest from `res` (the kernels ask for lanes 0..V-1 in order).
// simd128_ groups are 16-byte packs of the argument type (groups of fewer
// lanes, the scalar tail and misaligned tables, are scalar code); the scalar
// form takes the thread's whole group, reduced in one pass when its elements
// share a reduction level.
template <class Tag> struct trig_kind;
template <> struct trig_kind<tag::sin_> { static constexpr int value = trig::SIN; };
template <> struct trig_kind<tag::cos_> { static constexpr int value = trig::COS; };
template <> struct trig_kind<tag::tan_> { static constexpr int value = trig::TAN; };
template <> struct trig_kind<tag::sinpi_> { static constexpr int value = trig::SINPI; };
template <> struct trig_kind<tag::cospi_> { static constexpr int value = trig::COSPI; };
template <> struct trig_kind<tag::cot_> { static constexpr int value = trig::COT; };
template <> struct trig_kind<tag::tanpi_> { static constexpr int value = trig::TANPI; };
template <> struct trig_kind<tag::cotpi_> { static constexpr int value = trig::COTPI; };
template <> struct trig_kind<tag::sind_> { static constexpr int value = trig::SIND; };
template <> struct trig_kind<tag::cosd_> { static constexpr int value = trig::COSD; };
template <> struct trig_kind<tag::tand_> { static constexpr int value = trig::TAND; };
template <> struct trig_kind<tag::cotd_> { static constexpr int value = trig::COTD; };

template <class NodeTag, class Tag, bool SIMD, class A, int V> struct trig_regs {
  using N = node<NodeTag, A>;
  using T = typename value_of<A>::type;
  static_assert(std::is_same<T, float>::value || std::is_same<T, double>::value,
                "trigonometric functors take float or double tables");
  static constexpr int PW = 16 / (int)sizeof(T);
  static constexpr int P = SIMD ? ((V % PW == 0) ? PW : 1) : V;
  regs<A, V> ra;
  mutable T res[V];
  template <bool S> __device__ __forceinline__ void load(const N& n, size_t i) { ra.template load<S>(n.a, i); }
  template <bool S> __device__ __forceinline__ void load_one(const N& n, size_t i, int l) { ra.template load_one<S>(n.a, i, l); }
  template <bool F> __device__ __forceinline__ T get(const N& n, int l) const {
    if (l % P == 0) {
      T a[P], y[P];
#pragma unroll
      for (int p = 0; p < P; ++p) a[p] = (T)ra.template get<F>(n.a, l + p);
      if constexpr (SIMD) trig::pack<trig_kind<Tag>::value, F, P>(a, y);
      else trig::scalar_group<trig_kind<Tag>::value, F, P>(a, y);
#pragma unroll
      for (int p = 0; p < P; ++p) res[l + p] = y[p];
    }
    return res[l];
  }
};
#define NT2CUDA_TRIG_REGS(TAG)                                                                     \
  template <class A, int V> struct regs<node<tag::TAG, A>, V> : trig_regs<tag::TAG, tag::TAG, false, A, V> {}; \
  template <class A, int V>                                                                        \
  struct regs<node<tag::simd128_<tag::TAG>, A>, V> : trig_regs<tag::simd128_<tag::TAG>, tag::TAG, true, A, V> {};
NT2CUDA_TRIG_REGS(sin_)
NT2CUDA_TRIG_REGS(cos_)
NT2CUDA_TRIG_REGS(tan_)
NT2CUDA_TRIG_REGS(sinpi_)
NT2CUDA_TRIG_REGS(cospi_)
NT2CUDA_TRIG_REGS(cot_)
NT2CUDA_TRIG_REGS(tanpi_)
NT2CUDA_TRIG_REGS(cotpi_)
NT2CUDA_TRIG_REGS(sind_)
NT2CUDA_TRIG_REGS(cosd_)
NT2CUDA_TRIG_REGS(tand_)
NT2CUDA_TRIG_REGS(cotd_)
#undef NT2CUDA_TRIG_REGS

// prefetch_terms(e, i): L2 prefetch of element i of every table read by e.
template <class T> __device__ __forceinline__ void prefetch_terms(const term<T>& t, size_t i) { mem::prefetch_l2(t.p + i); }
template <class T> __device__ __forceinline__ void prefetch_terms(const scal<T>&, size_t) {}
template <class Tag, class A> __device__ __forceinline__ void prefetch_terms(const node<Tag, A>& n, size_t i)
{ prefetch_terms(n.a, i); }
template <class Tag, class A, class B> __device__ __forceinline__ void prefetch_terms(const node<Tag, A, B>& n, size_t i)
{ prefetch_terms(n.a, i); prefetch_terms(n.b, i); }
template <class Tag, class A, class B, class C>
__device__ __forceinline__ void prefetch_terms(const node<Tag, A, B, C>& n, size_t i)
{ prefetch_terms(n.a, i); prefetch_terms(n.b, i); prefetch_terms(n.c, i); }

// ------------------------------------------------------------- programs
// Nodes that expand into long instruction sequences: every functor but the
// elementwise arithmetic, comparisons and selections.  A statement with
// several of them keeps too many temporaries live for two groups per thread
// (the unrolled kernels are held to 64 or 80 registers and spill), so its
// launches default to one group per thread per trip (`transform` below).
template <class Tag> struct light_tag { static constexpr bool value = false; };
#define NT2CUDA_LIGHT(TAG) template <> struct light_tag<tag::TAG> { static constexpr bool value = true; };
NT2CUDA_LIGHT(plus_) NT2CUDA_LIGHT(minus_) NT2CUDA_LIGHT(multiplies_) NT2CUDA_LIGHT(unary_minus_)
NT2CUDA_LIGHT(fma_) NT2CUDA_LIGHT(fnms_) NT2CUDA_LIGHT(sqr_) NT2CUDA_LIGHT(abs_) NT2CUDA_LIGHT(max_)
NT2CUDA_LIGHT(min_) NT2CUDA_LIGHT(adds_) NT2CUDA_LIGHT(subs_) NT2CUDA_LIGHT(selinc_) NT2CUDA_LIGHT(seldec_)
NT2CUDA_LIGHT(if_else_) NT2CUDA_LIGHT(if_zero_else_one_) NT2CUDA_LIGHT(is_less_) NT2CUDA_LIGHT(is_greater_)
NT2CUDA_LIGHT(is_less_equal_) NT2CUDA_LIGHT(is_greater_equal_) NT2CUDA_LIGHT(is_equal_)
NT2CUDA_LIGHT(is_not_equal_) NT2CUDA_LIGHT(oneminus_) NT2CUDA_LIGHT(minusone_) NT2CUDA_LIGHT(cast_)
NT2CUDA_LIGHT(trunc_u8_)
#undef NT2CUDA_LIGHT
template <class E> struct heavy_nodes { static constexpr int value = 0; };
template <class Tag, class... C> struct heavy_nodes<node<Tag, C...>> {
  static constexpr int value = (light_tag<Tag>::value ? 0 : 1) + (0 + ... + heavy_nodes<C>::value);
};

// prog<A0, A...>: the assigns of one statement, evaluated per index in order.
template <class... As> struct prog;
template <> struct prog<> {};
template <class A0, class... As> struct prog<A0, As...> { A0 head; prog<As...> tail; };

template <class... As> __host__ __device__ inline prog<As...> make_prog(As... as);
template <> __host__ __device__ inline prog<> make_prog() { return prog<>{}; }
template <class A0, class... As> __host__ __device__ inline prog<A0, As...> make_prog(A0 a0, As... as)
{
  return prog<A0, As...>{a0, make_prog(as...)};
}

// Lane count: enough lanes that the smallest element type moves 16 bytes.
template <class P> struct prog_min_elem;
template <> struct prog_min_elem<prog<>> { static constexpr int value = 1 << 20; };
template <class T, class E, class... As> struct prog_min_elem<prog<assign<T, E>, As...>> {
  static constexpr int a = min_elem<E>::value < (int)sizeof(T) ? min_elem<E>::value : (int)sizeof(T);
  static constexpr int b = prog_min_elem<prog<As...>>::value;
  static constexpr int value = a < b ? a : b;
};
template <class P> struct prog_heavy;
template <> struct prog_heavy<prog<>> { static constexpr int value = 0; };
template <class T, class E, class... As> struct prog_heavy<prog<assign<T, E>, As...>> {
  static constexpr int value = heavy_nodes<E>::value + prog_heavy<prog<As...>>::value;
};
template <class P> struct base_lanes {
  static constexpr int m = prog_min_elem<P>::value;
  static constexpr int value = m >= 16 ? 1 : 16 / m;
};

// L2 prefetch of element i of every table a program reads.
template <class... As> __device__ __forceinline__ void prefetch_prog(const prog<As...>&, size_t) {}
template <class T, class E, class... As>
__device__ __forceinline__ void prefetch_prog(const prog<assign<T, E>, As...>& p, size_t i)
{
  prefetch_terms(p.head.e, i);
  prefetch_prog(p.tail, i);
}

template <class P, int V> struct pregs;
template <int V> struct pregs<prog<>, V> {
  template <bool S> __device__ __forceinline__ void load(const prog<>&, size_t) {}
  template <bool F> __device__ __forceinline__ void compute_store(const prog<>&, size_t) {}
};
template <class T, class E, class... As, int V> struct pregs<prog<assign<T, E>, As...>, V> {
  using P = prog<assign<T, E>, As...>;
  regs<E, V> r;
  pregs<prog<As...>, V> rest;
  template <bool S> __device__ __forceinline__ void load(const P& p, size_t i) {
    r.template load<S>(p.head.e, i);
    rest.template load<S>(p.tail, i);
  }
  template <bool F> __device__ __forceinline__ void compute_store(const P& p, size_t i) {
    T out[V];
#pragma unroll
    for (int l = 0; l < V; ++l) out[l] = (T)r.template get<F>(p.head.e, l);
    mem::store_vec<T, V>(p.head.out, i, out);
    rest.template compute_store<F>(p.tail, i);
  }
};

// ---------------------------------------------------------- the kernel
// Persistent grid-stride transform.  Each thread owns groups of V contiguous
// elements and keeps U groups in flight per trip: all terminals of all
// assigns of a group are loaded before any of its outputs is stored, which
// is NT2's order for tie() statements.  The n % V tail is done one element
// per thread by the first threads of the grid.
// Unrolled variants ask the compiler for enough resident blocks that the
// extra groups in flight are not paid for with occupancy.
template <int U> struct transform_min_blocks { static constexpr int value = U == 1 ? 1 : (U == 2 ? 4 : 3); };

template <bool F, int V, int U, class P>
__global__ void __launch_bounds__(256, transform_min_blocks<U>::value) k_transform(P p, size_t n)
{
  const size_t ngroups = n / V;
  const size_t T = (size_t)gridDim.x * blockDim.x;
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  // while the previous grid drains, have the L2 fetch this thread's first U groups
#pragma unroll
  for (int u = 0; u < U; ++u)
    if (tid + (size_t)u * T < ngroups) prefetch_prog(p, (tid + (size_t)u * T) * V);
  nt2cuda::mem::pdl_begin();
  size_t g = tid;
#pragma unroll 1
  for (; g + (size_t)(U - 1) * T < ngroups; g += (size_t)U * T) {
    pregs<P, V> r[U];
#pragma unroll
    for (int u = 0; u < U; ++u) r[u].template load<true>(p, (g + (size_t)u * T) * V);
#pragma unroll
    for (int u = 0; u < U; ++u) r[u].template compute_store<F>(p, (g + (size_t)u * T) * V);
  }
#pragma unroll 1
  for (; g < ngroups; g += T) {
    pregs<P, V> r;
    r.template load<true>(p, g * V);
    r.template compute_store<F>(p, g * V);
  }
  const size_t tail0 = ngroups * V;
  if (tid < n - tail0) {
    pregs<P, 1> r;
    r.template load<false>(p, tail0 + tid);
    r.template compute_store<F>(p, tail0 + tid);
  }
}

}  // namespace nt2cuda
