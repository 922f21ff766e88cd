// nt2/sdk/cuda/eval.hpp -- the GB300 evaluation site of NT2.
//
// NT2 picks the backend that evaluates table statements by stacking
// dispatch sites at compile time (BOOST_DISPATCH_COMBINE_SITE,
// modules/boost/dispatch/include/boost/dispatch/functor/forward.hpp:84-98);
// OpenMP is one such site (modules/arch/openmp/include/nt2/sdk/openmp/shared_memory.hpp:17-25).
// This header adds cuda_eval_ on top of the stack and gives it NT2's three
// evaluation overloads:
//   transform_(out, in, range)              elementwise statements, tie excluded
//   inner_fold_(out, in, neutral, bop, uop) sum/prod/max/min along the first dims
//   outer_fold_(out, in, neutral, bop, uop) the same along a later dimension
// (modules/arch/shared_memory/include/nt2/core/functions/shared_memory/{transform,inner_fold,outer_fold}.hpp).
// Each lowers the Proto tree onto the nt2cuda expression nodes
// (nt2cuda/table_lowering.hpp) and runs it through nt2cuda/site.hpp: one
// fused kernel per statement, built by nvcc for sm_103a.  A statement with a
// functor, a leaf or a reduction that has no device form does not match the
// overload's condition, so Boost.Dispatch selects the parent site's overload
// (OpenMP or scalar) at compile time; nothing is decided at run time.
//
// Use: compile the NT2 translation unit with nvcc (-std=c++17,
// -gencode arch=compute_103a,code=sm_103a, -I <this repo>/include
// -I <this repo>/nt2_gb300/csrc), define NT2_HAS_CUDA_EVAL, include this
// header after NT2's own, and give tables device memory (NT2's container
// with an allocator over nt2cuda_alloc, or managed memory).  Failures raise
// nt2cuda::site::error.
#ifndef NT2_SDK_CUDA_EVAL_HPP_INCLUDED
#define NT2_SDK_CUDA_EVAL_HPP_INCLUDED

#include <stdexcept>
#include <string>
#include <type_traits>
#include <boost/dispatch/functor/forward.hpp>
#include <boost/proto/core.hpp>
#include <nt2/core/functions/transform.hpp>
#include <nt2/core/functions/inner_fold.hpp>
#include <nt2/core/functions/outer_fold.hpp>
#include <nt2/include/functions/numel.hpp>
#include "nt2cuda/site.hpp"

namespace nt2 { namespace tag
{
  template<typename Site> struct cuda_eval_ : Site
  {
    typedef Site parent;
  };
} }

// ------------------------------------------------ Proto tree access
namespace nt2cuda { namespace lowering
{
  template <class E>
  struct tree_access<E, typename std::enable_if<boost::proto::is_expr<E>::value>::type>
  {
    static constexpr bool terminal = boost::proto::arity_of<E>::value == 0;
    typedef typename boost::proto::tag_of<E>::type tag;
    static constexpr int arity = (int)boost::proto::arity_of<E>::value;
    template <int N> static auto& child(E& e) { return boost::proto::child_c<N>(e); }
    static auto& value(E& e) { return boost::proto::value(e); }
  };

  // the statement's output: a table terminal of float or double
  template <class Out> struct site_output
    : std::integral_constant<bool, boost::proto::arity_of<Out>::value == 0 &&
                                   (std::is_same<typename Out::value_type, float>::value ||
                                    std::is_same<typename Out::value_type, double>::value)> {};

  template <class Out, class In> struct site_accepts
    : std::integral_constant<bool, site_output<Out>::value && lowerable<In>::value> {};

  // the reduction tag carried by NT2's Uop functor (boost::dispatch::functor<Tag, Site>)
  template <class F> struct functor_tag { typedef void type; };
  template <template <class, class> class Fn, class Tag, class S> struct functor_tag<Fn<Tag, S> > { typedef Tag type; };

  template <class Out, class In, class Uop> struct site_accepts_fold
    : std::integral_constant<bool, site_accepts<Out, In>::value &&
                                   nt2cuda::site::site_fold<fold_of<typename functor_tag<Uop>::type>::value>::value> {};
} }

namespace nt2cuda { namespace site
{
  struct error : std::runtime_error
  {
    error(const char* where, cudaError_t e) : std::runtime_error(std::string(where) + ": " + cudaGetErrorString(e)) {}
  };
  inline void check(cudaError_t e, const char* where) { if (e != cudaSuccess) throw error(where, e); }
} }

#ifdef NT2_HAS_CUDA_EVAL
BOOST_DISPATCH_COMBINE_SITE( nt2::tag::cuda_eval_<tag::cpu_> )

namespace nt2 { namespace ext
{
  // out(range) = in(range): one fused kernel
  BOOST_DISPATCH_IMPLEMENT_IF ( transform_, (nt2::tag::cuda_eval_<Site>)
                              , (Out)(In)(Site)(Range)
                              , (nt2cuda::lowering::site_accepts<Out, In>)
                              , ((ast_<Out, nt2::container::domain>))
                                ((ast_<In, nt2::container::domain>))
                                (unspecified_<Range>)
                              )
  {
    typedef void result_type;
    BOOST_FORCEINLINE result_type operator()(Out& out, In& in, Range range) const
    {
      typedef typename Out::value_type T;
      nt2cuda::site::check(nt2cuda::site::transform<T>(out.data(), in, range.first, range.second),
                           "nt2 cuda_eval_ transform");
    }
  };

  // in viewed as (inner, outer): out(j) = uop over i of in(i, j)
  BOOST_DISPATCH_IMPLEMENT_IF ( inner_fold_, (nt2::tag::cuda_eval_<Site>)
                              , (Out)(In)(Neutral)(Bop)(Uop)(Site)
                              , (nt2cuda::lowering::site_accepts_fold<Out, In, Uop>)
                              , ((ast_<Out, nt2::container::domain>))
                                ((ast_<In, nt2::container::domain>))
                                (unspecified_<Neutral>)
                                (unspecified_<Bop>)
                                (unspecified_<Uop>)
                              )
  {
    typedef void result_type;
    BOOST_FORCEINLINE result_type
    operator()(Out& out, In& in, Neutral const&, Bop const&, Uop const&) const
    {
      typedef typename Out::value_type T;
      typedef typename nt2cuda::lowering::functor_tag<Uop>::type tag_t;
      typename In::extent_type ext = in.extent();
      const std::size_t inner = boost::fusion::at_c<0>(ext);
      const std::size_t outer = nt2::numel(boost::fusion::pop_front(ext));
      nt2cuda::site::check(nt2cuda::site::inner_fold<nt2cuda::lowering::fold_of<tag_t>::value, T>(out.data(), in,
                                                                                                  inner, outer),
                           "nt2 cuda_eval_ inner_fold");
    }
  };

  // in viewed as (lo, inner, hi): out(l, k) = uop over m of in(l, m, k)
  BOOST_DISPATCH_IMPLEMENT_IF ( outer_fold_, (nt2::tag::cuda_eval_<Site>)
                              , (Out)(In)(Neutral)(Bop)(Uop)(Site)
                              , (nt2cuda::lowering::site_accepts_fold<Out, In, Uop>)
                              , ((ast_<Out, nt2::container::domain>))
                                ((ast_<In, nt2::container::domain>))
                                (unspecified_<Neutral>)
                                (unspecified_<Bop>)
                                (unspecified_<Uop>)
                              )
  {
    typedef void result_type;
    BOOST_FORCEINLINE result_type
    operator()(Out& out, In& in, Neutral const&, Bop const&, Uop const&) const
    {
      typedef typename Out::value_type T;
      typedef typename nt2cuda::lowering::functor_tag<Uop>::type tag_t;
      typename In::extent_type ext = in.extent();
      const std::size_t lo = boost::fusion::at_c<0>(ext);
      const std::size_t inner = boost::fusion::at_c<1>(ext);
      const std::size_t hi = boost::fusion::at_c<2>(ext);
      nt2cuda::site::check(nt2cuda::site::outer_fold<nt2cuda::lowering::fold_of<tag_t>::value, T>(out.data(), in,
                                                                                                  lo, inner, hi),
                           "nt2 cuda_eval_ outer_fold");
    }
  };
} }
#endif

#endif
