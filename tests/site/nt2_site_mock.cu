// nt2_site_mock.cu -- the NT2 evaluation site driven by a mock of NT2's
// expression trees (test program).
//
// NT2's trees are Boost.Proto expressions: inner nodes carry NT2's functor
// tags, leaves hold a table (a memory container with value_type and data())
// or a splatted scalar.  Boost is not available here, so this program builds
// trees of the same shape from the real tag types (forward-declared by
// nt2cuda/table_lowering.hpp), specializes tree_access<> for them as
// nt2/sdk/cuda/eval.hpp does for Proto, and calls the site operations that
// eval.hpp's transform_ / inner_fold_ / outer_fold_ overloads call.
//
// Subcommands (tables are raw little-endian files):
//   saxpy n alpha x y out                  out = fma(alpha, X, Y)   (after NT2's a*b+c -> fma rewrite)
//   bs n r v S K T call put                the Black-Scholes call/put statements, one tree each
//   sdot n x y out                         sum(reshape(X*Y, of_size(n,1)))  (inner_fold_)
//   rowsum rows cols A out                 sum(A, 2)                        (outer_fold_, hi = 1)
//   range n begin size alpha x y out       transform_ over [begin, begin+size) only
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <tuple>
#include <vector>
#include "nt2cuda/site.hpp"

namespace mock {
template <class T> struct container {        // NT2's memory container: value_type, data()
  typedef T value_type;
  T* p;
  T* data() { return p; }
};
template <class V> struct leaf { V v; };     // a terminal
template <class Tag, class... C> struct expr { std::tuple<C...> kids; };

template <class Tag, class... C> expr<Tag, C...> mk(C... c) { return expr<Tag, C...>{std::tuple<C...>(c...)}; }
template <class T> leaf<container<T>> tab(T* p) { return leaf<container<T>>{container<T>{p}}; }
template <class T> leaf<T> sc(T v) { return leaf<T>{v}; }
}  // namespace mock

namespace nt2cuda { namespace lowering {
template <class V> struct tree_access<mock::leaf<V>> {
  static constexpr bool terminal = true;
  typedef void tag;
  static constexpr int arity = 0;
  static V& value(mock::leaf<V>& e) { return e.v; }
};
template <class Tag, class... C> struct tree_access<mock::expr<Tag, C...>> {
  static constexpr bool terminal = false;
  typedef Tag tag;
  static constexpr int arity = (int)sizeof...(C);
  template <int N> static auto& child(mock::expr<Tag, C...>& e) { return std::get<N>(e.kids); }
};
} }

namespace bt = boost::simd::tag;
namespace nt = nt2::tag;
using mock::mk;
using mock::sc;
using mock::tab;

template <class T> static T* upload(const char* path, size_t n)
{
  std::vector<T> h(n);
  FILE* f = std::fopen(path, "rb");
  if (!f || std::fread(h.data(), sizeof(T), n, f) != n) { std::fprintf(stderr, "cannot read %s\n", path); std::exit(2); }
  std::fclose(f);
  T* d = nullptr;
  if (cudaMalloc(&d, n * sizeof(T) + 16) != cudaSuccess) std::exit(3);
  cudaMemcpy(d, h.data(), n * sizeof(T), cudaMemcpyHostToDevice);
  return d;
}
template <class T> static T* device(size_t n)
{
  T* d = nullptr;
  if (cudaMalloc(&d, n * sizeof(T) + 16) != cudaSuccess) std::exit(3);
  cudaMemset(d, 0, n * sizeof(T));
  return d;
}
template <class T> static void download(const char* path, const T* d, size_t n)
{
  std::vector<T> h(n);
  cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost);
  FILE* f = std::fopen(path, "wb");
  std::fwrite(h.data(), sizeof(T), n, f);
  std::fclose(f);
}
static void ok(cudaError_t e, const char* what)
{
  if (e != cudaSuccess) { std::fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e)); std::exit(4); }
}

int main(int argc, char** argv)
{
  if (argc < 3) return 1;
  const char* cmd = argv[1];
  if (!std::strcmp(cmd, "saxpy") || !std::strcmp(cmd, "range")) {
    const bool range = !std::strcmp(cmd, "range");
    const size_t n = std::strtoull(argv[2], nullptr, 10);
    int a = 3;
    const size_t begin = range ? std::strtoull(argv[a++], nullptr, 10) : 0;
    const size_t size = range ? std::strtoull(argv[a++], nullptr, 10) : n;
    const float alpha = std::strtof(argv[a++], nullptr);
    float* x = upload<float>(argv[a++], n);
    float* y = upload<float>(argv[a++], n);
    // Y = alpha*X + Y, as NT2 evaluates it after rewriting a*b+c into fma(a,b,c)
    auto st = mk<bt::fma_>(sc(alpha), tab(x), tab(y));
    static_assert(nt2cuda::lowering::lowerable<decltype(st)>::value, "saxpy tree must lower");
    ok(nt2cuda::site::transform<float>(y, st, begin, size), "saxpy");
    download(argv[a], y, n);
    return 0;
  }
  if (!std::strcmp(cmd, "bs")) {
    const size_t n = std::strtoull(argv[2], nullptr, 10);
    const float r = std::strtof(argv[3], nullptr), v = std::strtof(argv[4], nullptr);
    float* S = upload<float>(argv[5], n);
    float* K = upload<float>(argv[6], n);
    float* T = upload<float>(argv[7], n);
    float* call = device<float>(n);
    float* put = device<float>(n);
    // da = sqrt(T); vda = v*da; d1 = (log(S/K) + fma(sqr(v),0.5,r)*T)/vda (the sum rewritten to fma);
    // d2 = d1 - vda; e = K*exp(-r*T); call = fnms(e, normcdf(d2), S*normcdf(d1));
    // put = fnms(S, normcdf(-d1), e*normcdf(-d2))
    auto vda = mk<bt::multiplies_>(sc(v), mk<bt::sqrt_>(tab(T)));
    auto c = mk<bt::fma_>(mk<bt::sqr_>(sc(v)), sc(0.5f), sc(r));
    auto d1 = mk<bt::divides_>(mk<bt::fma_>(c, tab(T), mk<nt::log_>(mk<bt::divides_>(tab(S), tab(K)))), vda);
    auto d2 = mk<bt::minus_>(d1, vda);
    auto e = mk<bt::multiplies_>(tab(K), mk<nt::exp_>(mk<bt::multiplies_>(mk<bt::unary_minus_>(sc(r)), tab(T))));
    auto call_st = mk<bt::fnms_>(e, mk<nt::normcdf_>(d2), mk<bt::multiplies_>(tab(S), mk<nt::normcdf_>(d1)));
    auto put_st = mk<bt::fnms_>(tab(S), mk<nt::normcdf_>(mk<bt::unary_minus_>(d1)),
                                mk<bt::multiplies_>(e, mk<nt::normcdf_>(mk<bt::unary_minus_>(d2))));
    ok(nt2cuda::site::transform<float>(call, call_st, 0, n), "bs call");
    ok(nt2cuda::site::transform<float>(put, put_st, 0, n), "bs put");
    download(argv[8], call, n);
    download(argv[9], put, n);
    return 0;
  }
  if (!std::strcmp(cmd, "sdot")) {
    const size_t n = std::strtoull(argv[2], nullptr, 10);
    float* x = upload<float>(argv[3], n);
    float* y = upload<float>(argv[4], n);
    float* out = device<float>(1);
    // globalsum(X*Y) = sum(colvect(X*Y))(1): the fold receives reshape(colvect(X*Y), of_size(n, 1))
    auto in = mk<nt::reshape_>(mk<nt::colvect_>(mk<bt::multiplies_>(tab(x), tab(y))), sc(0));
    static_assert(nt2cuda::lowering::lowerable<decltype(in)>::value, "sdot tree must lower");
    ok(nt2cuda::site::inner_fold<nt2cuda::lowering::fold_of<bt::sum_>::value, float>(out, in, n, 1), "sdot");
    download(argv[5], out, 1);
    return 0;
  }
  if (!std::strcmp(cmd, "rowsum")) {
    const size_t rows = std::strtoull(argv[2], nullptr, 10), cols = std::strtoull(argv[3], nullptr, 10);
    float* A = upload<float>(argv[4], rows * cols);
    float* out = device<float>(rows);
    auto in = mk<nt::reshape_>(tab(A), sc(0));
    ok(nt2cuda::site::outer_fold<nt2cuda::lowering::fold_of<bt::sum_>::value, float>(out, in, rows, cols, 1),
       "rowsum");
    download(argv[5], out, rows);
    return 0;
  }
  // a tree with a functor that has no device form is not lowerable: the site
  // would leave it to the parent site
  struct no_device_form_;
  static_assert(!nt2cuda::lowering::lowerable<decltype(mk<no_device_form_>(tab((float*)nullptr)))>::value,
                "unknown functors must not lower");
  return 1;
}
