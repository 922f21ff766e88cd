// nt2cuda/table.hpp -- NT2's table / expression front end, evaluated on the GPU.
//
// User code written against nt2::table compiles unchanged against this
// header (compiled by nvcc, -std=c++17, with include/ and nt2_gb300/csrc/ on
// the include path) once `nt2` is aliased to `nt2cuda`:
//
//     nt2cuda::table<float> X(nt2cuda::of_size(n)), Y(nt2cuda::of_size(n));
//     for (std::size_t i = 1; i <= n; ++i) X(i) = Y(i) = float(i - 1);
//     Y = alpha * X + Y;                          // one fused kernel
//     float s = nt2cuda::globalsum(X * Y);        // fused fold
//     nt2cuda::tie(call, put) = nt2cuda::tie(e1, e2);
//
// Mirrors (paths relative to the NT2 source tree):
//   table container      modules/core/container/table/include/nt2/core/container/table/table.hpp:26-121
//   assignment           modules/core/sdk/include/nt2/core/container/dsl/expression.hpp:161-191
//   tie()                modules/core/container/table/include/nt2/core/functions/expr/tie.hpp:40-182
//   globalsum / sum      modules/core/reduction/include/nt2/core/functions/globalsum.hpp:75-88,
//                        modules/core/reduction/include/nt2/dsl/functions/reduction/run.hpp:30-104
//
// Residency: a table owns a device buffer in HBM and a host mirror that is
// created on first element access.  Element access (1-based, column-major,
// as NT2) moves the data to the host once and marks the device copy stale;
// the next evaluation that reads the table uploads it once.  Evaluations run
// on the table's stream (nt2cuda::set_stream) and, like NT2's operator=,
// return with the results ready unless nt2cuda::set_synchronous(false).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#include <cstring>
#include <istream>
#include <ostream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>
#include "nt2cuda/expr.cuh"
#include "nt2cuda/fold_launch.cuh"
#include "nt2cuda/scan_launch.cuh"
#include "nt2cuda/launch.cuh"

namespace nt2cuda {

// ------------------------------------------------------------ settings
struct eval_settings {
  cudaStream_t stream = nullptr;
  bool synchronous = true;
  bool fused = false;       // hardware FMA for NT2's fma/fnms/horner steps
  bool compensated = true;  // compensated FP32 folds
};
inline eval_settings& settings() { static thread_local eval_settings s; return s; }
inline void set_stream(cudaStream_t s) { settings().stream = s; }
inline void set_synchronous(bool b) { settings().synchronous = b; }
inline void set_fused(bool b) { settings().fused = b; }
inline void set_compensated(bool b) { settings().compensated = b; }

struct error : std::runtime_error {
  explicit error(const std::string& w, cudaError_t e)
      : std::runtime_error(w + ": " + cudaGetErrorString(e)), code(e) {}
  cudaError_t code;
};
inline void check(cudaError_t e, const char* where)
{
  if (e != cudaSuccess) throw error(where, e);
}

// ------------------------------------------------------------ of_size
struct of_size_ {
  size_t d[2] = {0, 1};
  size_t numel() const { return d[0] * d[1]; }
};
inline of_size_ of_size(size_t n) { of_size_ s; s.d[0] = n; s.d[1] = 1; return s; }
inline of_size_ of_size(size_t h, size_t w) { of_size_ s; s.d[0] = h; s.d[1] = w; return s; }

template <class E> struct xpr;   // lazy expression
template <class T> class table;

// ------------------------------------------------------------- table
template <class T> class table {
 public:
  using value_type = T;
  table() = default;
  explicit table(of_size_ s) { resize(s); }
  table(const table& o) { *this = o; }
  table(table&& o) noexcept { swap(o); }
  template <class E> table(const xpr<E>& x) { *this = x; }
  ~table() { release(); }

  table& operator=(table&& o) noexcept { swap(o); return *this; }
  table& operator=(const table& o)
  {
    if (this == &o) return *this;
    resize(o.extent());
    if (!numel()) return *this;
    o.sync_device();
    check(cudaMemcpyAsync(d_, o.d_, numel() * sizeof(T), cudaMemcpyDeviceToDevice, settings().stream),
          "table copy");
    dev_valid_ = true;
    host_valid_ = false;
    finish();
    return *this;
  }
  template <class E> table& operator=(const xpr<E>& x);

  void resize(of_size_ s)
  {
    if (s.d[0] == sz_.d[0] && s.d[1] == sz_.d[1]) return;
    release();
    sz_ = s;
    if (numel()) check(cudaMalloc(&d_, numel() * sizeof(T)), "table alloc");
    dev_valid_ = true;
    host_valid_ = false;
  }

  size_t numel() const { return sz_.numel(); }
  of_size_ extent() const { return sz_; }
  size_t height() const { return sz_.d[0]; }
  size_t width() const { return sz_.d[1]; }

  // 1-based element access (host mirror)
  T& operator()(size_t i) { sync_host(); dev_valid_ = false; return h_[i - 1]; }
  T& operator()(size_t i, size_t j) { return (*this)(i + (j - 1) * sz_.d[0]); }
  T operator()(size_t i) const { sync_host(); return h_[i - 1]; }
  T operator()(size_t i, size_t j) const { return (*this)(i + (j - 1) * sz_.d[0]); }

  // device pointer with the device copy current
  T* device() { sync_device(); host_valid_ = false; return d_; }
  const T* device() const { sync_device(); return d_; }
  void mark_device_written() { dev_valid_ = true; host_valid_ = false; }
  // replace the contents from host data (numel() elements, column-major);
  // the device copy is refreshed by the next sync_device()
  void assign_host(std::vector<T>&& data)
  {
    if (data.size() != numel()) throw std::invalid_argument("assign_host: element count differs from numel()");
    h_ = std::move(data);
    host_valid_ = true;
    dev_valid_ = numel() == 0;
  }
  // the host mirror, current after sync_host()
  const std::vector<T>& host() const { sync_host(); return h_; }

  void sync_host() const
  {
    if (host_valid_) return;
    h_.resize(numel());
    if (numel()) {
      check(cudaMemcpyAsync(h_.data(), d_, numel() * sizeof(T), cudaMemcpyDeviceToHost, settings().stream), "d2h");
      check(cudaStreamSynchronize(settings().stream), "d2h sync");
    }
    host_valid_ = true;
  }
  void sync_device() const
  {
    if (dev_valid_) return;
    if (numel())
      check(cudaMemcpyAsync(d_, h_.data(), numel() * sizeof(T), cudaMemcpyHostToDevice, settings().stream), "h2d");
    // h2d from pageable memory is staged before return; the host mirror stays valid
    dev_valid_ = true;
  }

 private:
  void release()
  {
    if (d_) cudaFree(d_);
    d_ = nullptr;
    h_.clear();
    sz_ = of_size_{};
    dev_valid_ = true;
    host_valid_ = false;
  }
  void swap(table& o) noexcept
  {
    std::swap(d_, o.d_);
    std::swap(sz_, o.sz_);
    h_.swap(o.h_);
    std::swap(dev_valid_, o.dev_valid_);
    std::swap(host_valid_, o.host_valid_);
  }
  static void finish()
  {
    if (settings().synchronous) check(cudaStreamSynchronize(settings().stream), "evaluation");
  }

  T* d_ = nullptr;
  of_size_ sz_{};
  mutable std::vector<T> h_;
  mutable bool dev_valid_ = true;
  mutable bool host_valid_ = false;
  template <class> friend class table;
  friend struct detail_front;
};

// ----------------------------------------------------------- expressions
// xpr<E> holds the device tree E plus the element count it evaluates over.
template <class E> struct xpr {
  E e;
  of_size_ size;
  using value_type = typename value_of<E>::type;
};

template <class X> struct is_table : std::false_type {};
template <class T> struct is_table<table<T>> : std::true_type {};
template <class X> struct is_xpr : std::false_type {};
template <class E> struct is_xpr<xpr<E>> : std::true_type {};
template <class X> constexpr bool is_operand_v =
    is_table<std::decay_t<X>>::value || is_xpr<std::decay_t<X>>::value;

// operand -> (tree, size)
template <class T> inline term<T> tree_of(const table<T>& t) { return term<T>{t.device()}; }
template <class E> inline E tree_of(const xpr<E>& x) { return x.e; }
template <class T> inline of_size_ size_of(const table<T>& t) { return t.extent(); }
template <class E> inline of_size_ size_of(const xpr<E>& x) { return x.size; }
template <class X> struct elem_of;
template <class T> struct elem_of<table<T>> { using type = T; };
template <class E> struct elem_of<xpr<E>> { using type = typename value_of<E>::type; };

inline of_size_ common_size(of_size_ a, of_size_ b)
{
  if (a.numel() != b.numel()) throw std::invalid_argument("nt2cuda: operand sizes differ");
  return a;
}

// scalar operand, converted to the element type of the other side
template <class V, class S> inline scal<V> scalar_as(S s) { return scal<V>{(V)s}; }

template <class Tag, class A> inline auto make_unary(const A& a)
{
  auto t = tree_of(a);
  return xpr<node<Tag, decltype(t)>>{node<Tag, decltype(t)>{t}, size_of(a)};
}

template <class Tag, class A, class B> inline auto make_binary(const A& a, const B& b)
{
  if constexpr (is_operand_v<A> && is_operand_v<B>) {
    auto ta = tree_of(a);
    auto tb = tree_of(b);
    return xpr<node<Tag, decltype(ta), decltype(tb)>>{node<Tag, decltype(ta), decltype(tb)>{ta, tb},
                                                      common_size(size_of(a), size_of(b))};
  } else if constexpr (is_operand_v<A>) {
    using V = typename elem_of<std::decay_t<A>>::type;
    auto ta = tree_of(a);
    auto tb = scalar_as<V>(b);
    return xpr<node<Tag, decltype(ta), decltype(tb)>>{node<Tag, decltype(ta), decltype(tb)>{ta, tb}, size_of(a)};
  } else {
    using V = typename elem_of<std::decay_t<B>>::type;
    auto ta = scalar_as<V>(a);
    auto tb = tree_of(b);
    return xpr<node<Tag, decltype(ta), decltype(tb)>>{node<Tag, decltype(ta), decltype(tb)>{ta, tb}, size_of(b)};
  }
}

template <class X, class V> inline auto tree_or_scalar(const X& x)
{
  if constexpr (is_operand_v<X>) return tree_of(x); else return scal<V>{(V)x};
}

template <class Tag, class A, class B, class C> inline auto make_ternary(const A& a, const B& b, const C& c)
{
  // element type: first table/expression operand among a, b, c
  using V = typename std::conditional_t<is_operand_v<A>, elem_of<std::decay_t<A>>,
            std::conditional_t<is_operand_v<B>, elem_of<std::decay_t<B>>, elem_of<std::decay_t<C>>>>::type;
  auto ta = tree_or_scalar<A, V>(a);
  auto tb = tree_or_scalar<B, V>(b);
  auto tc = tree_or_scalar<C, V>(c);
  of_size_ sz{};
  bool have = false;
  auto take = [&](const auto& x) {
    if constexpr (is_operand_v<std::decay_t<decltype(x)>>) {
      sz = have ? common_size(sz, size_of(x)) : size_of(x);
      have = true;
    }
  };
  take(a); take(b); take(c);
  using N = node<Tag, decltype(ta), decltype(tb), decltype(tc)>;
  return xpr<N>{N{ta, tb, tc}, sz};
}

#define NT2CUDA_BINOP(OP, TAG)                                                          \
  template <class A, class B, std::enable_if_t<is_operand_v<A> || is_operand_v<B>, int> = 0> \
  inline auto operator OP(const A& a, const B& b) { return make_binary<tag::TAG>(a, b); }
NT2CUDA_BINOP(+, plus_)
NT2CUDA_BINOP(-, minus_)
NT2CUDA_BINOP(*, multiplies_)
NT2CUDA_BINOP(/, divides_)
NT2CUDA_BINOP(<, is_less_)
NT2CUDA_BINOP(>, is_greater_)
NT2CUDA_BINOP(<=, is_less_equal_)
NT2CUDA_BINOP(>=, is_greater_equal_)
NT2CUDA_BINOP(==, is_equal_)
NT2CUDA_BINOP(!=, is_not_equal_)
#undef NT2CUDA_BINOP

template <class A, std::enable_if_t<is_operand_v<A>, int> = 0>
inline auto operator-(const A& a) { return make_unary<tag::unary_minus_>(a); }

#define NT2CUDA_FN1(NAME, TAG)                                                          \
  template <class A, std::enable_if_t<is_operand_v<A>, int> = 0>                        \
  inline auto NAME(const A& a) { return make_unary<tag::TAG>(a); }
NT2CUDA_FN1(exp, exp_)
NT2CUDA_FN1(log, log_)
NT2CUDA_FN1(exp2, exp2_)
NT2CUDA_FN1(exp10, exp10_)
NT2CUDA_FN1(log2, log2_)
NT2CUDA_FN1(log10, log10_)
NT2CUDA_FN1(expm1, expm1_)
NT2CUDA_FN1(log1p, log1p_)
NT2CUDA_FN1(sin, sin_)
NT2CUDA_FN1(cos, cos_)
NT2CUDA_FN1(tan, tan_)
NT2CUDA_FN1(sinpi, sinpi_)
NT2CUDA_FN1(cospi, cospi_)
NT2CUDA_FN1(cot, cot_)
NT2CUDA_FN1(tanpi, tanpi_)
NT2CUDA_FN1(cotpi, cotpi_)
NT2CUDA_FN1(sind, sind_)
NT2CUDA_FN1(cosd, cosd_)
NT2CUDA_FN1(tand, tand_)
NT2CUDA_FN1(cotd, cotd_)
NT2CUDA_FN1(asin, asin_)
NT2CUDA_FN1(acos, acos_)
NT2CUDA_FN1(atan, atan_)
NT2CUDA_FN1(sinh, sinh_)
NT2CUDA_FN1(cosh, cosh_)
NT2CUDA_FN1(tanh, tanh_)
NT2CUDA_FN1(atanh, atanh_)
NT2CUDA_FN1(acosh, acosh_)
NT2CUDA_FN1(asinh, asinh_)
NT2CUDA_FN1(coth, coth_)
NT2CUDA_FN1(sinhc, sinhc_)
NT2CUDA_FN1(cbrt, cbrt_)
NT2CUDA_FN1(sqrt1pm1, sqrt1pm1_)
NT2CUDA_FN1(exprecneg, exprecneg_)
NT2CUDA_FN1(exprecnegc, exprecnegc_)
NT2CUDA_FN1(expx2, expx2_)
NT2CUDA_FN1(realsqrt, sqrt_)
NT2CUDA_FN1(reallog, log_)
NT2CUDA_FN1(sqrt, sqrt_)
NT2CUDA_FN1(sqr, sqr_)
NT2CUDA_FN1(erfc, erfc_)
NT2CUDA_FN1(normcdf, normcdf_)
NT2CUDA_FN1(fastnormcdf, fastnormcdf_)
NT2CUDA_FN1(abs, abs_)
NT2CUDA_FN1(rec, rec_)
NT2CUDA_FN1(oneminus, oneminus_)
NT2CUDA_FN1(minusone, minusone_)
#undef NT2CUDA_FN1

#define NT2CUDA_FN2(NAME, TAG)                                                          \
  template <class A, class B, std::enable_if_t<is_operand_v<A> || is_operand_v<B>, int> = 0> \
  inline auto NAME(const A& a, const B& b) { return make_binary<tag::TAG>(a, b); }
NT2CUDA_FN2(max, max_)
NT2CUDA_FN2(atan2, atan2_)
NT2CUDA_FN2(pow, pow_)
NT2CUDA_FN2(realpow, pow_)
NT2CUDA_FN2(pow_abs, pow_abs_)
NT2CUDA_FN2(logspace_add, logspace_add_)
NT2CUDA_FN2(logspace_sub, logspace_sub_)
NT2CUDA_FN2(expx2, expx2s_)
NT2CUDA_FN2(atan2d, atan2d_)
NT2CUDA_FN2(nbd_atan2, nbd_atan2_)
NT2CUDA_FN2(hypot, hypot_)
NT2CUDA_FN2(min, min_)
NT2CUDA_FN2(adds, adds_)
NT2CUDA_FN2(subs, subs_)
NT2CUDA_FN2(selinc, selinc_)
NT2CUDA_FN2(seldec, seldec_)
#undef NT2CUDA_FN2

// Trigonometric functors NT2 composes from the ones above, as one fused statement each
// (modules/core/trigonometric/include/nt2/trigonometric/functions/generic/<name>.hpp; asec:
// simd/common/asec.hpp).
#define NT2CUDA_COMPOSED(NAME, EXPR)                                                    \
  template <class A, std::enable_if_t<is_operand_v<A>, int> = 0>                        \
  inline auto NAME(const A& a) { return EXPR; }
NT2CUDA_COMPOSED(indeg, make_unary<tag::indeg_>(a))
NT2CUDA_COMPOSED(inrad, make_unary<tag::inrad_>(a))
NT2CUDA_COMPOSED(csc, rec(sin(a)))
NT2CUDA_COMPOSED(sec, rec(cos(a)))
NT2CUDA_COMPOSED(cscpi, make_binary<tag::cscpi_nan_>(a, rec(sinpi(a))))
NT2CUDA_COMPOSED(secpi, make_binary<tag::secpi_nan_>(a, rec(cospi(a))))
NT2CUDA_COMPOSED(cscd, cscpi(make_unary<tag::oneo_180_mul_>(a)))
NT2CUDA_COMPOSED(acot, atan(rec(a)))
NT2CUDA_COMPOSED(asind, indeg(asin(a)))
NT2CUDA_COMPOSED(acosd, indeg(acos(a)))
NT2CUDA_COMPOSED(atand, indeg(atan(a)))
NT2CUDA_COMPOSED(asinpi, make_unary<tag::invpi_mul_>(asin(a)))
NT2CUDA_COMPOSED(acospi, make_unary<tag::invpi_mul_>(acos(a)))
NT2CUDA_COMPOSED(atanpi, make_unary<tag::invpi_mul_>(atan(a)))
NT2CUDA_COMPOSED(acsc, asin(rec(a)))
NT2CUDA_COMPOSED(acscd, indeg(acsc(a)))
NT2CUDA_COMPOSED(asec, make_unary<tag::pio2_minus_>(acsc(a)))
NT2CUDA_COMPOSED(asecd, indeg(asec(a)))
NT2CUDA_COMPOSED(secd, rec(make_unary<tag::nan_if_zero_>(cosd(a))))
NT2CUDA_COMPOSED(sinc, make_binary<tag::sinc_fix_>(a, sin(a) / a))
NT2CUDA_COMPOSED(sincpi, make_binary<tag::sinc_fix_>(a, make_unary<tag::invpi_mul_>(sinpi(a) / a)))
NT2CUDA_COMPOSED(sech, rec(cosh(a)))
NT2CUDA_COMPOSED(csch, rec(sinh(a)))
NT2CUDA_COMPOSED(acoth, atanh(rec(a)))
NT2CUDA_COMPOSED(asech, acosh(rec(a)))
NT2CUDA_COMPOSED(acsch, asinh(rec(a)))
NT2CUDA_COMPOSED(fast_sin, (make_unary<tag::fast_<0, 0>>(a)))
NT2CUDA_COMPOSED(fast_cos, (make_unary<tag::fast_<1, 0>>(a)))
NT2CUDA_COMPOSED(fast_tan, (make_unary<tag::fast_<2, 0>>(a)))
NT2CUDA_COMPOSED(fast_cot, (make_unary<tag::fast_<3, 0>>(a)))
NT2CUDA_COMPOSED(fast_sinpi, (make_unary<tag::fast_<0, 1>>(a)))
NT2CUDA_COMPOSED(fast_cospi, (make_unary<tag::fast_<1, 1>>(a)))
NT2CUDA_COMPOSED(fast_tanpi, (make_unary<tag::fast_<2, 1>>(a)))
NT2CUDA_COMPOSED(fast_cotpi, (make_unary<tag::fast_<3, 1>>(a)))
NT2CUDA_COMPOSED(fast_sind, (make_unary<tag::fast_<0, 2>>(a)))
NT2CUDA_COMPOSED(fast_cosd, (make_unary<tag::fast_<1, 2>>(a)))
NT2CUDA_COMPOSED(fast_tand, (make_unary<tag::fast_<2, 2>>(a)))
NT2CUDA_COMPOSED(fast_cotd, (make_unary<tag::fast_<3, 2>>(a)))
NT2CUDA_COMPOSED(proper_tanpi, make_unary<tag::proper_tanpi_>(a))
#undef NT2CUDA_COMPOSED

#define NT2CUDA_FN3(NAME, TAG)                                                          \
  template <class A, class B, class C,                                                  \
            std::enable_if_t<is_operand_v<A> || is_operand_v<B> || is_operand_v<C>, int> = 0> \
  inline auto NAME(const A& a, const B& b, const C& c) { return make_ternary<tag::TAG>(a, b, c); }
NT2CUDA_FN3(fma, fma_)
NT2CUDA_FN3(fnms, fnms_)
NT2CUDA_FN3(if_else, if_else_)
#undef NT2CUDA_FN3

// cast<R>(x): the elements of x converted to R, as nt2::cast
// (nt2/operator/functions/container/cast.hpp:133-150).
template <class R, class A, std::enable_if_t<is_operand_v<A>, int> = 0> inline auto cast(const A& a)
{
  auto t = tree_of(a);
  using N = node<tag::cast_, decltype(t), scal<R>>;
  return xpr<N>{N{t, scal<R>{R(0)}}, size_of(a)};
}

// if_zero_else_one(c): the result has the element type of the compared operands.
template <class E> inline auto if_zero_else_one(const xpr<E>& c)
{
  using R = typename value_of<std::decay_t<decltype(c.e.a)>>::type;
  using N = node<tag::if_zero_else_one_, E, scal<R>>;
  return xpr<N>{N{c.e, scal<R>{R(0)}}, c.size};
}

// ------------------------------------------------------- evaluation
template <class T> template <class E> table<T>& table<T>::operator=(const xpr<E>& x)
{
  // NT2 resizes the left-hand side to the right-hand side's extent before
  // evaluating (modules/core/base/include/nt2/dsl/functions/elementwise/run.hpp:32).
  // The same number of elements in another shape keeps the buffer (the tree
  // may read this table: its device pointer was captured when the tree was
  // built); another number of elements gets a new buffer (an elementwise
  // tree of that size cannot read this table).
  if (x.size.d[0] != sz_.d[0] || x.size.d[1] != sz_.d[1]) {
    if (x.size.numel() == numel()) sz_ = x.size;
    else resize(x.size);
  }
  T* out = device();
  auto p = make_prog(assign<T, E>{out, x.e});
  cudaError_t e = settings().fused ? transform<true>(p, numel(), settings().stream)
                                   : transform<false>(p, numel(), settings().stream);
  check(e, "transform");
  check(cudaGetLastError(), "transform launch");
  mark_device_written();
  finish();
  return *this;
}

// ------------------------------------------------------------------ tie
template <class... Ts> struct tie_lhs {
  std::tuple<table<Ts>&...> outs;

  template <class... Es> tie_lhs& operator=(const std::tuple<xpr<Es>...>& rhs)
  {
    static_assert(sizeof...(Es) == sizeof...(Ts), "tie: arity mismatch");
    assign_all(rhs, std::index_sequence_for<Ts...>{});
    return *this;
  }

 private:
  template <class R, size_t... I> void assign_all(const R& rhs, std::index_sequence<I...>)
  {
    const size_t n = std::get<0>(rhs).size.numel();
    // outputs are sized first; their device pointers are the assign targets
    int dummy[] = {(prepare(std::get<I>(outs), n), 0)...};
    (void)dummy;
    auto p = make_prog(assign<typename std::remove_reference_t<decltype(std::get<I>(outs))>::value_type,
                              std::decay_t<decltype(std::get<I>(rhs).e)>>{std::get<I>(outs).device(),
                                                                          std::get<I>(rhs).e}...);
    cudaError_t e = settings().fused ? transform<true>(p, n, settings().stream)
                                     : transform<false>(p, n, settings().stream);
    check(e, "tie transform");
    check(cudaGetLastError(), "tie launch");
    int dummy2[] = {(std::get<I>(outs).mark_device_written(), 0)...};
    (void)dummy2;
    if (settings().synchronous) check(cudaStreamSynchronize(settings().stream), "tie");
  }
  template <class T> static void prepare(table<T>& t, size_t n)
  {
    if (t.numel() != n) t.resize(of_size(n));
  }
};

template <class... Ts> inline tie_lhs<Ts...> tie(table<Ts>&... ts) { return tie_lhs<Ts...>{{ts...}}; }
template <class... Es> inline std::tuple<xpr<Es>...> tie(const xpr<Es>&... xs) { return std::tuple<xpr<Es>...>(xs...); }

// ------------------------------------------------------------ reductions
template <class X> inline auto as_xpr(const X& x)
{
  if constexpr (is_table<std::decay_t<X>>::value) {
    using T = typename std::decay_t<X>::value_type;
    return xpr<term<T>>{term<T>{x.device()}, x.extent()};
  } else {
    return x;
  }
}

// globalsum(X): the sum of every element, on the host
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto globalsum(const X& x)
{
  auto e = as_xpr(x);
  using V = typename decltype(e)::value_type;
  using A = std::conditional_t<std::is_floating_point<V>::value, V, double>;
  static_assert(std::is_same<A, float>::value || std::is_same<A, double>::value, "globalsum: float or double");
  // the device scalar lives in the stream's own scratch (allocated by the
  // first reduction on the stream, reused after): no allocation per call
  cudaStream_t s = settings().stream;
  void* scratch = nullptr;
  check(stream_scratch(s, sizeof(A), &scratch, kResultSlot), "globalsum scratch");
  A* d = static_cast<A*>(scratch);
  cudaError_t err = (std::is_same<A, float>::value && settings().compensated)
                        ? fold::inner_fold<fold::op_sum<true>, A>(e.e, e.size.numel(), 1, d, s)
                        : fold::inner_fold<fold::op_sum<false>, A>(e.e, e.size.numel(), 1, d, s);
  A r = 0;
  if (err == cudaSuccess) err = cudaMemcpyAsync(&r, d, sizeof(A), cudaMemcpyDeviceToHost, s);
  if (err == cudaSuccess) err = cudaStreamSynchronize(s);
  check(err, "globalsum");
  return (V)r;
}

// sum(A, dim) for a 2-D table (dim 1: column sums, dim 2: row sums), as NT2's
// reduction run_assign picks inner_fold or outer_fold.
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto sum(const X& x, int dim = 1)
{
  auto e = as_xpr(x);
  using V = typename decltype(e)::value_type;
  const size_t rows = e.size.d[0], cols = e.size.d[1];
  cudaStream_t s = settings().stream;
  if (dim == 1) {
    table<V> out(of_size(1, cols));
    cudaError_t err = settings().compensated && std::is_same<V, float>::value
                          ? fold::inner_fold<fold::op_sum<true>, V>(e.e, rows, cols, out.device(), s)
                          : fold::inner_fold<fold::op_sum<false>, V>(e.e, rows, cols, out.device(), s);
    check(err, "sum(A,1)");
    out.mark_device_written();
    if (settings().synchronous) check(cudaStreamSynchronize(s), "sum");
    return out;
  }
  table<V> out(of_size(rows, 1));
  cudaError_t err = settings().compensated && std::is_same<V, float>::value
                        ? fold::outer_fold<fold::op_sum<true>, V>(e.e, rows, cols, out.device(), s)
                        : fold::outer_fold<fold::op_sum<false>, V>(e.e, rows, cols, out.device(), s);
  check(err, "sum(A,2)");
  out.mark_device_written();
  if (settings().synchronous) check(cudaStreamSynchronize(s), "sum");
  return out;
}

// ------------------------------------------- the other reductions and scans
// NT2's reductions along a dimension (1: one value per column, 2: one per row)
// or over every element (the global* forms), on the fold kernels with the
// operation policies of nt2cuda/fold.cuh
// (nt2/core/functions/expr/{asum1,asum2,norm2,mean,var,stdev}.hpp,
//  boost/simd/reduction/functions/{maximum,minimum,prod,all,any,none}.hpp),
// and the cumulative functions on the scan kernels of nt2cuda/scan.cuh
// (boost/simd/swar/functions/{cumsum,cumprod,cummax,cummin}.hpp).
namespace detail_table {
template <class X> using value_t = typename decltype(as_xpr(std::declval<X>()))::value_type;
template <class V, int FIN = fold::FIN_NONE>
using sum_op = std::conditional_t<std::is_same<V, float>::value, fold::op_sum<true, FIN>, fold::op_sum<false, FIN>>;

template <class Op, class X> inline auto reduce_dim(const X& x, int dim, const char* what)
{
  auto e = as_xpr(x);
  using V = typename decltype(e)::value_type;
  using O = fold::out_of<Op, V>;
  const size_t rows = e.size.d[0], cols = e.size.d[1];
  cudaStream_t s = settings().stream;
  table<O> out(dim == 1 ? of_size(1, cols) : of_size(rows, 1));
  cudaError_t err = dim == 1 ? fold::inner_fold<Op, V>(e.e, rows, cols, out.device(), s)
                             : fold::outer_fold<Op, V>(e.e, rows, cols, out.device(), s);
  check(err, what);
  out.mark_device_written();
  if (settings().synchronous) check(cudaStreamSynchronize(s), what);
  return out;
}

template <class Op, class X> inline auto reduce_all(const X& x, const char* what)
{
  auto e = as_xpr(x);
  using V = typename decltype(e)::value_type;
  using O = fold::out_of<Op, V>;
  cudaStream_t s = settings().stream;
  void* scratch = nullptr;                       // the stream's result slot, as globalsum
  check(stream_scratch(s, sizeof(O), &scratch, kResultSlot), what);
  O* d = static_cast<O*>(scratch);
  cudaError_t err = fold::inner_fold<Op, V>(e.e, e.size.numel(), 1, d, s);
  O r{};
  if (err == cudaSuccess) err = cudaMemcpyAsync(&r, d, sizeof(O), cudaMemcpyDeviceToHost, s);
  if (err == cudaSuccess) err = cudaStreamSynchronize(s);
  check(err, what);
  return r;
}

template <class Op, class X> inline auto scan_dim(const X& x, int dim, const char* what)
{
  using V = value_t<X>;
  table<V> in;
  const V* src;
  of_size_ sz;
  if constexpr (is_table<std::decay_t<X>>::value) {
    src = x.device();
    sz = x.extent();
  } else {                    // an expression is evaluated into a table first, as NT2's scan reads it
    in = x;
    src = in.device();
    sz = in.extent();
  }
  table<V> out(sz);
  cudaStream_t s = settings().stream;
  check(scan::scan_dim<Op, V>(src, out.device(), sz.d[0], sz.numel() / (sz.d[0] ? sz.d[0] : 1), dim, s), what);
  out.mark_device_written();
  if (settings().synchronous) check(cudaStreamSynchronize(s), what);
  return out;
}
}  // namespace detail_table

template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto asum1(const X& x, int dim = 1)
{ return detail_table::reduce_dim<detail_table::sum_op<detail_table::value_t<X>>>(abs(x), dim, "asum1"); }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto globalasum1(const X& x)
{ return detail_table::reduce_all<detail_table::sum_op<detail_table::value_t<X>>>(abs(x), "globalasum1"); }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto asum2(const X& x, int dim = 1)
{ return detail_table::reduce_dim<detail_table::sum_op<detail_table::value_t<X>>>(sqr(x), dim, "asum2"); }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto globalasum2(const X& x)
{ return detail_table::reduce_all<detail_table::sum_op<detail_table::value_t<X>>>(sqr(x), "globalasum2"); }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto norm2(const X& x, int dim = 1)
{ return detail_table::reduce_dim<detail_table::sum_op<detail_table::value_t<X>, fold::FIN_SQRT>>(sqr(x), dim, "norm2"); }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto globalnorm2(const X& x)
{ return detail_table::reduce_all<detail_table::sum_op<detail_table::value_t<X>, fold::FIN_SQRT>>(sqr(x), "globalnorm2"); }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto mean(const X& x, int dim = 1)
{ return detail_table::reduce_dim<detail_table::sum_op<detail_table::value_t<X>, fold::FIN_MEAN>>(x, dim, "mean"); }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto globalmean(const X& x)
{ return detail_table::reduce_all<detail_table::sum_op<detail_table::value_t<X>, fold::FIN_MEAN>>(x, "globalmean"); }
// var(A, w, dim) / stdev(A, w, dim): w = 0 normalises by n - 1, w = 1 by n
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto var(const X& x, int w = 0, int dim = 1)
{
  return w ? detail_table::reduce_dim<fold::op_moments<true, false>>(x, dim, "var")
           : detail_table::reduce_dim<fold::op_moments<false, false>>(x, dim, "var");
}
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto stdev(const X& x, int w = 0, int dim = 1)
{
  return w ? detail_table::reduce_dim<fold::op_moments<true, true>>(x, dim, "stdev")
           : detail_table::reduce_dim<fold::op_moments<false, true>>(x, dim, "stdev");
}
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto globalvar(const X& x, int w = 0)
{
  return w ? detail_table::reduce_all<fold::op_moments<true, false>>(x, "globalvar")
           : detail_table::reduce_all<fold::op_moments<false, false>>(x, "globalvar");
}
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto globalstdev(const X& x, int w = 0)
{
  return w ? detail_table::reduce_all<fold::op_moments<true, true>>(x, "globalstdev")
           : detail_table::reduce_all<fold::op_moments<false, true>>(x, "globalstdev");
}
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto maximum(const X& x, int dim = 1)
{ return detail_table::reduce_dim<fold::op_val<0>>(x, dim, "maximum"); }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto globalmax(const X& x)
{ return detail_table::reduce_all<fold::op_val<0>>(x, "globalmax"); }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto minimum(const X& x, int dim = 1)
{ return detail_table::reduce_dim<fold::op_val<1>>(x, dim, "minimum"); }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto globalmin(const X& x)
{ return detail_table::reduce_all<fold::op_val<1>>(x, "globalmin"); }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto prod(const X& x, int dim = 1)
{ return detail_table::reduce_dim<fold::op_val<2>>(x, dim, "prod"); }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto globalprod(const X& x)
{ return detail_table::reduce_all<fold::op_val<2>>(x, "globalprod"); }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto all(const X& x, int dim = 1)
{ return detail_table::reduce_dim<fold::op_logic<false>>(x, dim, "all"); }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline bool globalall(const X& x)
{ return detail_table::reduce_all<fold::op_logic<false>>(x, "globalall") != 0; }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto any(const X& x, int dim = 1)
{ return detail_table::reduce_dim<fold::op_logic<true>>(x, dim, "any"); }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline bool globalany(const X& x)
{ return detail_table::reduce_all<fold::op_logic<true>>(x, "globalany") != 0; }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto none(const X& x, int dim = 1)
{ return detail_table::reduce_dim<fold::op_logic<true, true>>(x, dim, "none"); }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline bool globalnone(const X& x)
{ return detail_table::reduce_all<fold::op_logic<true, true>>(x, "globalnone") != 0; }

template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto cumsum(const X& x, int dim = 1)
{ return detail_table::scan_dim<detail_table::sum_op<detail_table::value_t<X>>>(x, dim, "cumsum"); }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto cumprod(const X& x, int dim = 1)
{ return detail_table::scan_dim<fold::op_val<2>>(x, dim, "cumprod"); }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto cummax(const X& x, int dim = 1)
{ return detail_table::scan_dim<fold::op_val<3>>(x, dim, "cummax"); }
template <class X, std::enable_if_t<is_operand_v<X>, int> = 0> inline auto cummin(const X& x, int dim = 1)
{ return detail_table::scan_dim<fold::op_val<4>>(x, dim, "cummin"); }

// ----------------------------------------------------------- table I/O
// NT2 serializes a table as its extent followed by its numel() elements
// (modules/core/container/table/include/nt2/core/container/io/serialization.hpp:48-83,
// written through a Boost.Serialization archive).  save/load write the same two
// fields in a fixed little-endian layout that needs no Boost:
//   8 bytes   "NT2TABLE"
//   4 bytes   element size in bytes      4 bytes  element kind: 'f', 'i' or 'u'
//   8 bytes   extent 1 (rows)            8 bytes  extent 2 (columns)
//   rows * columns elements, column-major
// save is a host<->device sync point: the device copy is brought to the host
// mirror first.  load fills the host mirror and marks the device copy stale,
// so the first evaluation that reads the table copies it up.
namespace detail_table {
template <class T> constexpr uint32_t kind_of()
{
  return std::is_floating_point<T>::value ? 'f' : (std::is_signed<T>::value ? 'i' : 'u');
}
inline void put64(std::ostream& os, uint64_t v)
{
  unsigned char b[8];
  for (int i = 0; i < 8; ++i) b[i] = (unsigned char)(v >> (8 * i));
  os.write((const char*)b, 8);
}
inline void put32(std::ostream& os, uint32_t v)
{
  unsigned char b[4];
  for (int i = 0; i < 4; ++i) b[i] = (unsigned char)(v >> (8 * i));
  os.write((const char*)b, 4);
}
inline uint64_t get64(std::istream& is)
{
  unsigned char b[8] = {};
  is.read((char*)b, 8);
  uint64_t v = 0;
  for (int i = 7; i >= 0; --i) v = (v << 8) | b[i];
  return v;
}
inline uint32_t get32(std::istream& is)
{
  unsigned char b[4] = {};
  is.read((char*)b, 4);
  uint32_t v = 0;
  for (int i = 3; i >= 0; --i) v = (v << 8) | b[i];
  return v;
}
}  // namespace detail_table

template <class T> void save(std::ostream& os, const table<T>& t)
{
  static_assert(std::is_arithmetic<T>::value, "save: tables of numbers");
  const std::vector<T>& h = t.host();
  os.write("NT2TABLE", 8);
  detail_table::put32(os, (uint32_t)sizeof(T));
  detail_table::put32(os, detail_table::kind_of<T>());
  detail_table::put64(os, t.height());
  detail_table::put64(os, t.width());
  // elements in the host's byte order: little-endian on x86-64 and aarch64
  if (!h.empty()) os.write((const char*)h.data(), (std::streamsize)(h.size() * sizeof(T)));
  if (!os) throw std::runtime_error("nt2cuda::save: write failed");
}

template <class T> void load(std::istream& is, table<T>& t)
{
  static_assert(std::is_arithmetic<T>::value, "load: tables of numbers");
  char magic[8] = {};
  is.read(magic, 8);
  if (!is || std::memcmp(magic, "NT2TABLE", 8) != 0) throw std::runtime_error("nt2cuda::load: not a table file");
  const uint32_t size = detail_table::get32(is), kind = detail_table::get32(is);
  if (size != sizeof(T) || kind != detail_table::kind_of<T>())
    throw std::runtime_error("nt2cuda::load: element type differs from the table's");
  const uint64_t rows = detail_table::get64(is), cols = detail_table::get64(is);
  if (!is || (cols && rows > ~(uint64_t)0 / cols)) throw std::runtime_error("nt2cuda::load: bad extent");
  std::vector<T> data((size_t)(rows * cols));
  if (!data.empty()) is.read((char*)data.data(), (std::streamsize)(data.size() * sizeof(T)));
  if (!is) throw std::runtime_error("nt2cuda::load: file ends early");
  t.resize(of_size((size_t)rows, (size_t)cols));
  t.assign_host(std::move(data));
}

}  // namespace nt2cuda
