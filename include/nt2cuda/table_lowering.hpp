// nt2cuda/table_lowering.hpp -- lowering of an NT2 expression tree onto the
// device expression nodes of nt2cuda/expr.cuh.
//
// NT2 builds every table statement as a Boost.Proto tree whose inner nodes
// carry a functor tag (boost::simd::tag::plus_, nt2::tag::exp_, ...) and
// whose leaves are terminals holding a table or a scalar
// (modules/core/sdk/include/nt2/core/container/dsl/expression.hpp:161-191);
// its CPU backends evaluate that tree per index
// (modules/core/sdk/include/nt2/dsl/functions/generic/run.hpp:180-222,
//  modules/core/sdk/include/nt2/dsl/functions/container/terminal.hpp:28-198).
// The GPU site instead maps the whole tree, at compile time, onto one
// nt2cuda::node<> type and launches the fused kernel built for it.
//
// This header needs neither Boost nor NT2.  It names NT2's functor tags by
// forward declaration (they are plain structs in boost::simd::tag and
// nt2::tag, so the declarations agree with NT2's definitions), and it reads
// trees through one trait, tree_access<E>, that the caller specializes:
//   static constexpr bool terminal;           // a leaf?
//   using tag = ...;                          // inner node: NT2's functor tag
//   static constexpr int arity;               // inner node: 1, 2 or 3 children
//   template <int N> static auto& child(E&);  // inner node: the N-th child
//   static auto& value(E&);                   // leaf: the table or the scalar
// nt2/sdk/cuda/eval.hpp specializes it for Boost.Proto expressions
// (proto::tag_of, proto::arity_of, proto::child_c, proto::value); the tests
// specialize it for a mock tree of the same shape.
//
// A table leaf is anything with value_type and data() (NT2's memory
// containers, modules/core/sdk/include/nt2/sdk/memory/container.hpp:359-366,
// holding device memory under this site); it lowers to
// term<T>{data() + offset}.  An
// arithmetic leaf is a splatted scalar; it lowers to scal<S> with S the
// statement's element type, the type NT2 splats it to in a homogeneous
// statement.  A tree whose tags or leaves are not all covered is not
// lowerable, and the site leaves such statements to the next site (the CPU).
#pragma once
#include <stddef.h>
#include <type_traits>
#include <utility>
#include "nt2cuda/expr.cuh"

// ------------------------------------------------ NT2's functor tags
// modules/boost/simd/base/include/boost/simd/{operator,arithmetic,boolean,reduction}/functions/*.hpp
namespace boost { namespace simd { namespace tag {
struct plus_; struct minus_; struct multiplies_; struct divides_; struct unary_minus_;
struct fma_; struct fnms_; struct sqr_; struct sqrt_; struct rec_; struct abs_;
struct max_; struct min_; struct adds_; struct subs_; struct oneminus_; struct minusone_;
struct selinc_; struct seldec_; struct if_else_; struct if_zero_else_one_;
struct is_less_; struct is_greater_; struct is_less_equal_; struct is_greater_equal_;
struct is_equal_; struct is_not_equal_;
struct sum_; struct prod_; struct maximum_; struct minimum_; struct all_; struct any_;
} } }
// modules/core/{exponential,euler,statistics,trigonometric,hyperbolic}/include/nt2/*/functions/*.hpp
namespace nt2 { namespace tag {
struct exp_; struct log_; struct exp2_; struct exp10_; struct log2_; struct log10_; struct expm1_; struct log1p_;
struct erfc_; struct normcdf_; struct fastnormcdf_;
struct sin_; struct cos_; struct tan_; struct sinpi_; struct cospi_; struct cot_; struct tanpi_; struct cotpi_;
struct sind_; struct cosd_; struct tand_; struct cotd_; struct asin_; struct acos_; struct atan_; struct atan2_;
struct sinh_; struct cosh_; struct tanh_; struct asinh_; struct acosh_; struct atanh_; struct coth_; struct sinhc_;
struct pow_; struct pow_abs_; struct cbrt_; struct sqrt1pm1_; struct exprecneg_; struct exprecnegc_;
struct hypot_; struct logspace_add_; struct logspace_sub_;
struct reshape_; struct colvect_;
} }

namespace nt2cuda {
namespace lowering {

// ------------------------------------------ tag map (NT2 -> device)
// device_tag<NT2 tag>::type is the expr.cuh tag of the same functor; void
// when the functor has no device form here.
template <class NT2Tag> struct device_tag { using type = void; static constexpr int arity = -1; };
#define NT2CUDA_LOWER_TAG(NS, NAME, ARITY) \
  template <> struct device_tag<NS::tag::NAME> { using type = nt2cuda::tag::NAME; static constexpr int arity = ARITY; };
NT2CUDA_LOWER_TAG(boost::simd, plus_, 2)
NT2CUDA_LOWER_TAG(boost::simd, minus_, 2)
NT2CUDA_LOWER_TAG(boost::simd, multiplies_, 2)
NT2CUDA_LOWER_TAG(boost::simd, divides_, 2)
NT2CUDA_LOWER_TAG(boost::simd, unary_minus_, 1)
NT2CUDA_LOWER_TAG(boost::simd, fma_, 3)
NT2CUDA_LOWER_TAG(boost::simd, fnms_, 3)
NT2CUDA_LOWER_TAG(boost::simd, sqr_, 1)
NT2CUDA_LOWER_TAG(boost::simd, sqrt_, 1)
NT2CUDA_LOWER_TAG(boost::simd, rec_, 1)
NT2CUDA_LOWER_TAG(boost::simd, abs_, 1)
NT2CUDA_LOWER_TAG(boost::simd, max_, 2)
NT2CUDA_LOWER_TAG(boost::simd, min_, 2)
NT2CUDA_LOWER_TAG(boost::simd, adds_, 2)
NT2CUDA_LOWER_TAG(boost::simd, subs_, 2)
NT2CUDA_LOWER_TAG(boost::simd, oneminus_, 1)
NT2CUDA_LOWER_TAG(boost::simd, minusone_, 1)
NT2CUDA_LOWER_TAG(boost::simd, selinc_, 2)
NT2CUDA_LOWER_TAG(boost::simd, seldec_, 2)
NT2CUDA_LOWER_TAG(boost::simd, if_else_, 3)
NT2CUDA_LOWER_TAG(boost::simd, is_less_, 2)
NT2CUDA_LOWER_TAG(boost::simd, is_greater_, 2)
NT2CUDA_LOWER_TAG(boost::simd, is_less_equal_, 2)
NT2CUDA_LOWER_TAG(boost::simd, is_greater_equal_, 2)
NT2CUDA_LOWER_TAG(boost::simd, is_equal_, 2)
NT2CUDA_LOWER_TAG(boost::simd, is_not_equal_, 2)
NT2CUDA_LOWER_TAG(nt2, exp_, 1)
NT2CUDA_LOWER_TAG(nt2, log_, 1)
NT2CUDA_LOWER_TAG(nt2, exp2_, 1)
NT2CUDA_LOWER_TAG(nt2, exp10_, 1)
NT2CUDA_LOWER_TAG(nt2, log2_, 1)
NT2CUDA_LOWER_TAG(nt2, log10_, 1)
NT2CUDA_LOWER_TAG(nt2, expm1_, 1)
NT2CUDA_LOWER_TAG(nt2, log1p_, 1)
NT2CUDA_LOWER_TAG(nt2, erfc_, 1)
NT2CUDA_LOWER_TAG(nt2, normcdf_, 1)
NT2CUDA_LOWER_TAG(nt2, fastnormcdf_, 1)
NT2CUDA_LOWER_TAG(nt2, sin_, 1)
NT2CUDA_LOWER_TAG(nt2, cos_, 1)
NT2CUDA_LOWER_TAG(nt2, tan_, 1)
NT2CUDA_LOWER_TAG(nt2, sinpi_, 1)
NT2CUDA_LOWER_TAG(nt2, cospi_, 1)
NT2CUDA_LOWER_TAG(nt2, cot_, 1)
NT2CUDA_LOWER_TAG(nt2, tanpi_, 1)
NT2CUDA_LOWER_TAG(nt2, cotpi_, 1)
NT2CUDA_LOWER_TAG(nt2, sind_, 1)
NT2CUDA_LOWER_TAG(nt2, cosd_, 1)
NT2CUDA_LOWER_TAG(nt2, tand_, 1)
NT2CUDA_LOWER_TAG(nt2, cotd_, 1)
NT2CUDA_LOWER_TAG(nt2, asin_, 1)
NT2CUDA_LOWER_TAG(nt2, acos_, 1)
NT2CUDA_LOWER_TAG(nt2, atan_, 1)
NT2CUDA_LOWER_TAG(nt2, atan2_, 2)
NT2CUDA_LOWER_TAG(nt2, sinh_, 1)
NT2CUDA_LOWER_TAG(nt2, cosh_, 1)
NT2CUDA_LOWER_TAG(nt2, tanh_, 1)
NT2CUDA_LOWER_TAG(nt2, asinh_, 1)
NT2CUDA_LOWER_TAG(nt2, acosh_, 1)
NT2CUDA_LOWER_TAG(nt2, atanh_, 1)
NT2CUDA_LOWER_TAG(nt2, coth_, 1)
NT2CUDA_LOWER_TAG(nt2, sinhc_, 1)
NT2CUDA_LOWER_TAG(nt2, pow_, 2)
NT2CUDA_LOWER_TAG(nt2, pow_abs_, 2)
NT2CUDA_LOWER_TAG(nt2, cbrt_, 1)
NT2CUDA_LOWER_TAG(nt2, sqrt1pm1_, 1)
NT2CUDA_LOWER_TAG(nt2, exprecneg_, 1)
NT2CUDA_LOWER_TAG(nt2, exprecnegc_, 1)
NT2CUDA_LOWER_TAG(nt2, hypot_, 2)
NT2CUDA_LOWER_TAG(nt2, logspace_add_, 2)
NT2CUDA_LOWER_TAG(nt2, logspace_sub_, 2)
#undef NT2CUDA_LOWER_TAG

// if_zero_else_one(c) has no second operand in NT2; the device node takes
// the result type as a scalar operand (see table.hpp).
template <> struct device_tag<boost::simd::tag::if_zero_else_one_> {
  using type = nt2cuda::tag::if_zero_else_one_;
  static constexpr int arity = 1;
};

// Reshaping nodes around an elementwise tree (the folds receive
// reshape(input, of_size(...)), globalsum(X) folds colvect(X)) keep the
// column-major element order, so the lowering passes through them to their
// first child (modules/core/restructuring/include/nt2/core/functions/{reshape,colvect}.hpp).
template <class NT2Tag> struct transparent : std::false_type {};
template <> struct transparent<nt2::tag::reshape_> : std::true_type {};
template <> struct transparent<nt2::tag::colvect_> : std::true_type {};

// Reduction tags -> the fold's operation policy (nt2cuda/fold.cuh), for the
// inner_fold_ / outer_fold_ overloads: NT2 passes the reduction's functor as
// `Uop` (modules/core/reduction/include/nt2/dsl/functions/reduction/run.hpp:72-88).
enum fold_kind { FOLD_NONE = -1, FOLD_SUM = 0, FOLD_PROD = 1, FOLD_MAX = 2, FOLD_MIN = 3, FOLD_ALL = 4, FOLD_ANY = 5 };
template <class NT2Tag> struct fold_of { static constexpr int value = FOLD_NONE; };
template <> struct fold_of<boost::simd::tag::sum_> { static constexpr int value = FOLD_SUM; };
template <> struct fold_of<boost::simd::tag::prod_> { static constexpr int value = FOLD_PROD; };
template <> struct fold_of<boost::simd::tag::maximum_> { static constexpr int value = FOLD_MAX; };
template <> struct fold_of<boost::simd::tag::minimum_> { static constexpr int value = FOLD_MIN; };
template <> struct fold_of<boost::simd::tag::all_> { static constexpr int value = FOLD_ALL; };
template <> struct fold_of<boost::simd::tag::any_> { static constexpr int value = FOLD_ANY; };

// ------------------------------------------------------ tree access
template <class E, class Enable = void> struct tree_access;   // specialized by the front end

// a table leaf: value_type and data()
template <class V, class = void> struct is_table_value : std::false_type {};
template <class V>
struct is_table_value<V, std::void_t<typename V::value_type, decltype(std::declval<V&>().data())>> : std::true_type {};

template <class E> using access_of = tree_access<std::remove_cv_t<std::remove_reference_t<E>>>;

// ------------------------------------------------- lowerable trees
// lowered<E>::ok is true when every node and leaf of E has a device form.
template <class E, bool Leaf = access_of<E>::terminal> struct lowered;

template <class E> struct lowered<E, true> {
  using V = std::remove_cv_t<std::remove_reference_t<decltype(access_of<E>::value(std::declval<E&>()))>>;
  static constexpr bool ok = is_table_value<V>::value || std::is_arithmetic<V>::value;
};

template <class E, int N> struct child_ok {
  using C = std::remove_reference_t<decltype(access_of<E>::template child<N>(std::declval<E&>()))>;
  static constexpr bool value = lowered<C>::ok;
};

template <class E, int A> struct children_ok : std::false_type {};
template <class E> struct children_ok<E, 1> : std::integral_constant<bool, child_ok<E, 0>::value> {};
template <class E> struct children_ok<E, 2>
    : std::integral_constant<bool, child_ok<E, 0>::value && child_ok<E, 1>::value> {};
template <class E> struct children_ok<E, 3>
    : std::integral_constant<bool, child_ok<E, 0>::value && child_ok<E, 1>::value && child_ok<E, 2>::value> {};

template <class E, bool Through = transparent<typename access_of<E>::tag>::value> struct lowered_node {
  using DT = typename device_tag<typename access_of<E>::tag>::type;
  static constexpr bool ok = !std::is_void<DT>::value && device_tag<typename access_of<E>::tag>::arity == access_of<E>::arity &&
                             children_ok<E, access_of<E>::arity>::value;
};
template <class E> struct lowered_node<E, true> {
  static constexpr bool ok = child_ok<E, 0>::value;
};
template <class E> struct lowered<E, false> {
  static constexpr bool ok = lowered_node<E>::ok;
};

// The statement out = in is lowerable when its tree is.
template <class In> struct lowerable : std::integral_constant<bool, lowered<In>::ok> {};

// ------------------------------------------------------------ lower()
template <class S, class E> auto lower(E& e, size_t offset);

namespace detail {
template <class S, class E> auto lower_leaf(E& e, size_t offset)
{
  auto& v = access_of<E>::value(e);
  using V = std::remove_cv_t<std::remove_reference_t<decltype(v)>>;
  if constexpr (is_table_value<V>::value) {
    using T = typename V::value_type;
    return term<T>{static_cast<const T*>(v.data()) + offset};
  } else {
    return scal<S>{static_cast<S>(v)};
  }
}

template <class S, class E> auto lower_node(E& e, size_t offset)
{
  using A = access_of<E>;
  using DT = typename device_tag<typename A::tag>::type;
  if constexpr (transparent<typename A::tag>::value) {
    return lower<S>(A::template child<0>(e), offset);
  } else if constexpr (std::is_same<DT, nt2cuda::tag::if_zero_else_one_>::value) {
    auto c0 = lower<S>(A::template child<0>(e), offset);
    return node<DT, decltype(c0), scal<S>>{c0, scal<S>{S(0)}};
  } else if constexpr (A::arity == 1) {
    auto c0 = lower<S>(A::template child<0>(e), offset);
    return node<DT, decltype(c0)>{c0};
  } else if constexpr (A::arity == 2) {
    auto c0 = lower<S>(A::template child<0>(e), offset);
    auto c1 = lower<S>(A::template child<1>(e), offset);
    return node<DT, decltype(c0), decltype(c1)>{c0, c1};
  } else {
    auto c0 = lower<S>(A::template child<0>(e), offset);
    auto c1 = lower<S>(A::template child<1>(e), offset);
    auto c2 = lower<S>(A::template child<2>(e), offset);
    return node<DT, decltype(c0), decltype(c1), decltype(c2)>{c0, c1, c2};
  }
}
}  // namespace detail

// The device expression of the tree e, every table leaf advanced by `offset`
// elements (the start of the range NT2's transform_ hands the site).
template <class S, class E> auto lower(E& e, size_t offset)
{
  if constexpr (access_of<E>::terminal) return detail::lower_leaf<S>(e, offset);
  else return detail::lower_node<S>(e, offset);
}

}  // namespace lowering
}  // namespace nt2cuda
