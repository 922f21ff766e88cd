// demos.cu -- NT2's demo statements, written as NT2 user code against the
// nt2cuda table front end (namespace nt2 = nt2cuda).  Each subcommand reads
// its input tables from raw binary files, evaluates the reference demo's
// statements and writes the result tables, so a test can compare them with
// the oracle:
//   saxpy      demo/saxpy/nt2/saxpy_nt2.cpp:39-42
//   sdot       demo/sdot/nt2/sdot_nt2.cpp:35-38
//   bs         demo/blackscholes/nt2/blackandscholes_nt2.cpp:53-60
//   bs_merged  demo/blackscholes/nt2_merged/blackandscholes_nt2_merged.cpp:57-64
//   rgb2grey   demo/rgb2grey/nt2/rgb2grey_nt2.cpp:42-45 (float, and uint8 planes through nt2::cast)
//   rgb2yuv    demo/rgb2yuv/nt2/rgb2yuv_nt2.cpp:28-33
//   sigmadelta demo/sigmadelta/nt2/sigmadelta_nt2.cpp:37-58, 100-106
//   stats      NT2 reductions and cumulative functions of a table (mean, var,
//              maximum, asum1, cumsum along both dimensions, global* forms)
//   io         table files (nt2cuda::load / save): B = A*2 + 1 of a loaded table, saved
//   trig       trigonometric functors inside one statement and a fold:
//              y = sin(x) + cos(x)*tan(x*0.25f) + cospi(x)*sinpi(x), globalsum(sin(x))
//   pow        z = pow(x, y) + pow(y, 2.0f): pow with a table and with a scalar exponent;
//              w = cbrt(x) + logspace_add(x, y)
//   trigx      y = csc(x) + asind(x*1e-3f) + secpi(x): composed trigonometric functors;
//              w = cot(x) + sind(x) + tanpi(x*0.01f)
//   reshape    assignments that change the left-hand table's extent, and
//              repeated globalsum on one stream
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>
#include "nt2cuda/table.hpp"

namespace nt2 = nt2cuda;

template <class T> static std::vector<T> read_file(const char* path, size_t n)
{
  std::vector<T> v(n);
  FILE* f = std::fopen(path, "rb");
  if (!f || std::fread(v.data(), sizeof(T), n, f) != n) { std::fprintf(stderr, "cannot read %s\n", path); std::exit(2); }
  std::fclose(f);
  return v;
}

template <class T> static void load(nt2::table<T>& t, const std::vector<T>& v)
{
  for (std::size_t i = 1; i <= t.numel(); ++i) t(i) = v[i - 1];
}

template <class T> static void write_table(const char* path, const nt2::table<T>& t)
{
  FILE* f = std::fopen(path, "wb");
  for (std::size_t i = 1; i <= t.numel(); ++i) { T x = t(i); std::fwrite(&x, sizeof(T), 1, f); }
  std::fclose(f);
}

// the five statements of the demo's do_work, one table assignment each
template <class Pixel>
static void do_work(Pixel& bkg, const Pixel& fr, Pixel& var, Pixel& diff_img, Pixel& mul_img, Pixel& out)
{
  typename Pixel::value_type zero = 0;
  bkg = nt2::selinc(bkg < fr, nt2::seldec(bkg > fr, bkg));
  diff_img = nt2::max(bkg, fr) - nt2::min(bkg, fr);
  mul_img = nt2::adds(nt2::adds(diff_img, diff_img), diff_img);
  var = nt2::if_else(diff_img != zero, nt2::selinc(var < mul_img, nt2::seldec(var > mul_img, var)), var);
  out = nt2::if_zero_else_one(diff_img < var);
}

int main(int argc, char** argv)
{
  if (argc < 3) { std::fprintf(stderr, "usage: demos <cmd> <n> files...\n"); return 2; }
  std::string cmd = argv[1];
  const std::size_t n = std::strtoull(argv[2], nullptr, 10);
  if (cmd == "saxpy") {                                   // in: x y ; out: y
    typedef float T;
    T alpha = 2.5f;
    nt2::table<T> X(nt2::of_size(n)), Y(nt2::of_size(n));
    load(X, read_file<T>(argv[3], n));
    load(Y, read_file<T>(argv[4], n));
    Y = alpha * X + Y;
    write_table(argv[5], Y);
  } else if (cmd == "sdot") {                             // in: x y ; prints the sum
    typedef float T;
    nt2::table<T> X(nt2::of_size(n)), Y(nt2::of_size(n));
    load(X, read_file<T>(argv[3], n));
    load(Y, read_file<T>(argv[4], n));
    T res = nt2::globalsum(X * Y);
    std::printf("%.9e\n", (double)res);
  } else if (cmd == "bs" || cmd == "bs_merged") {         // in: S X T r v ; out: R
    typedef float T;
    nt2::table<T> Sa(nt2::of_size(n)), Xa(nt2::of_size(n)), Ta(nt2::of_size(n)), ra(nt2::of_size(n)),
        va(nt2::of_size(n)), R(nt2::of_size(n));
    load(Sa, read_file<T>(argv[3], n));
    load(Xa, read_file<T>(argv[4], n));
    load(Ta, read_file<T>(argv[5], n));
    load(ra, read_file<T>(argv[6], n));
    load(va, read_file<T>(argv[7], n));
    if (cmd == "bs") {
      nt2::table<T> da = nt2::sqrt(Ta);
      nt2::table<T> d1 = nt2::log(Sa / Xa) + (nt2::fma(nt2::sqr(va), T(0.5), ra) * Ta) / (va * da);
      nt2::table<T> d2 = nt2::fnms(va, da, d1);
      R = nt2::fnms(Xa * nt2::exp(-ra * Ta), nt2::fastnormcdf(d2), Sa * nt2::fastnormcdf(d1));
    } else {
      nt2::table<T> da(nt2::of_size(n)), d1(nt2::of_size(n)), d2(nt2::of_size(n));
      // every right-hand side reads the tables as they were before the statement, so da is
      // right after one evaluation, d1 after two, d2 after three and R after four (the demo
      // calls its operator() repeatedly)
      for (int rep = 0; rep < 4; ++rep)
        nt2::tie(da, d1, d2, R) = nt2::tie(nt2::sqrt(Ta),
                                           nt2::log(Sa / Xa) + (nt2::fma(nt2::sqr(va), T(0.5), ra) * Ta) / (va * da),
                                           nt2::fnms(va, da, d1),
                                           nt2::fnms(Xa * nt2::exp(-ra * Ta), nt2::fastnormcdf(d2),
                                                     Sa * nt2::fastnormcdf(d1)));
    }
    write_table(argv[8], R);
  } else if (cmd == "rgb2grey") {                         // in: r g b ; out: gr
    typedef float T;
    nt2::table<T> r(nt2::of_size(n)), g(nt2::of_size(n)), b(nt2::of_size(n)), gr(nt2::of_size(n));
    load(r, read_file<T>(argv[3], n));
    load(g, read_file<T>(argv[4], n));
    load(b, read_file<T>(argv[5], n));
    gr = T(0.3) * r + T(0.59) * g + T(0.11) * b;
    write_table(argv[6], gr);
  } else if (cmd == "rgb2grey_u8") {                      // in: r g b (uint8) ; out: gr (uint8)
    typedef unsigned char T;
    nt2::table<T> r(nt2::of_size(n)), g(nt2::of_size(n)), b(nt2::of_size(n)), gr(nt2::of_size(n));
    load(r, read_file<T>(argv[3], n));
    load(g, read_file<T>(argv[4], n));
    load(b, read_file<T>(argv[5], n));
    gr = nt2::cast<T>(0.3f * nt2::cast<float>(r) + 0.59f * nt2::cast<float>(g) + 0.11f * nt2::cast<float>(b));
    write_table(argv[6], gr);
  } else if (cmd == "rgb2yuv") {                          // in: r g b ; out: y u v
    typedef float K;
    nt2::table<K> r(nt2::of_size(n)), g(nt2::of_size(n)), b(nt2::of_size(n));
    nt2::table<K> y(nt2::of_size(n)), u(nt2::of_size(n)), v(nt2::of_size(n));
    load(r, read_file<K>(argv[3], n));
    load(g, read_file<K>(argv[4], n));
    load(b, read_file<K>(argv[5], n));
    y = K(0.299f) * r + K(0.587f) * g + K(0.114f) * b;
    u = K(0.492f) * (b - y);
    v = K(0.877f) * (r - y);
    write_table(argv[6], y);
    write_table(argv[7], u);
    write_table(argv[8], v);
  } else if (cmd == "stats") {                            // n = rows; argv[3] = cols; in: A ; out: 7 tables
    typedef float T;
    const std::size_t cols = std::strtoull(argv[3], nullptr, 10);
    nt2::table<T> A(nt2::of_size(n, cols));
    load(A, read_file<T>(argv[4], n * cols));
    nt2::table<T> m1 = nt2::mean(A, 1);
    nt2::table<T> v2 = nt2::var(A, 0, 2);
    nt2::table<T> x1 = nt2::maximum(A, 1);
    nt2::table<T> a2 = nt2::asum1(A, 2);
    nt2::table<T> c1 = nt2::cumsum(A, 1);
    nt2::table<T> c2 = nt2::cumsum(A, 2);
    nt2::table<T> g(nt2::of_size(4));
    g(1) = nt2::globalsum(A);
    g(2) = nt2::globalnorm2(A);
    g(3) = nt2::globalmax(A);
    g(4) = nt2::globalstdev(A);
    write_table(argv[5], m1);
    write_table(argv[6], v2);
    write_table(argv[7], x1);
    write_table(argv[8], a2);
    write_table(argv[9], c1);
    write_table(argv[10], c2);
    write_table(argv[11], g);
  } else if (cmd == "io") {                               // n unused; in: table file ; out: table file
    typedef double T;
    nt2::table<T> A, B;
    {
      std::ifstream in(argv[3], std::ios::binary);
      nt2::load(in, A);
    }
    B = A * T(2) + T(1);
    std::ofstream out(argv[4], std::ios::binary);
    nt2::save(out, B);
    std::printf("%zu %zu\n", B.height(), B.width());
  } else if (cmd == "trig") {                             // n; in: x ; out: y, [globalsum(sin(x))]
    typedef float T;
    nt2::table<T> x(nt2::of_size(n)), y, g(nt2::of_size(1));
    load(x, read_file<T>(argv[3], n));
    y = nt2::sin(x) + nt2::cos(x) * nt2::tan(x * T(0.25)) + nt2::cospi(x) * nt2::sinpi(x);
    g(1) = nt2::globalsum(nt2::sin(x));
    write_table(argv[4], y);
    write_table(argv[5], g);
  } else if (cmd == "pow") {                              // n; in: x y ; out: z w
    typedef float T;
    nt2::table<T> x(nt2::of_size(n)), y(nt2::of_size(n)), z, w;
    load(x, read_file<T>(argv[3], n));
    load(y, read_file<T>(argv[4], n));
    z = nt2::pow(x, y) + nt2::pow(y, T(2));
    w = nt2::cbrt(x) + nt2::logspace_add(x, y);
    write_table(argv[5], z);
    write_table(argv[6], w);
  } else if (cmd == "trigx") {                            // n; in: x ; out: y w
    typedef float T;
    nt2::table<T> x(nt2::of_size(n)), y, w;
    load(x, read_file<T>(argv[3], n));
    y = nt2::csc(x) + nt2::asind(x * T(1e-3)) + nt2::secpi(x);
    w = nt2::cot(x) + nt2::sind(x) + nt2::tanpi(x * T(0.01));
    write_table(argv[4], y);
    write_table(argv[5], w);
  } else if (cmd == "sigmadelta") {                       // n = pixels; argv[3] = frames; in: frames ; out: bkg var label
    typedef unsigned char T;
    const int nb_frames = std::atoi(argv[3]);
    std::vector<T> all = read_file<T>(argv[4], n * (std::size_t)nb_frames);
    std::vector<nt2::table<T>> frames((std::size_t)nb_frames);
    for (int k = 0; k < nb_frames; ++k) {
      frames[(std::size_t)k].resize(nt2::of_size(n));
      for (std::size_t i = 1; i <= n; ++i) frames[(std::size_t)k](i) = all[(std::size_t)k * n + i - 1];
    }
    nt2::table<T> image_variance(nt2::of_size(n)), diff_img(nt2::of_size(n)), mul_img(nt2::of_size(n)),
        background_img(nt2::of_size(n)), binary_label(nt2::of_size(n));
    for (std::size_t i = 1; i <= n; ++i) { image_variance(i) = 1; background_img(i) = frames[0](i); }
    for (int k = 1; k < nb_frames; ++k)
      do_work(background_img, frames[(std::size_t)k], image_variance, diff_img, mul_img, binary_label);
    write_table(argv[5], background_img);
    write_table(argv[6], image_variance);
    write_table(argv[7], binary_label);
  } else if (cmd == "reshape") {                          // n = rows; argv[3] = cols; in: A ; out: B1 B2 B3
    // NT2's assignment takes the right-hand side's extent (elementwise/run.hpp:32):
    // B = A*2+1 sizes B as A; B = At+1 (same elements, cols x rows) reshapes B in
    // place; B = C*3 (another size) reallocates it; globalsum twice on one stream.
    typedef float T;
    const std::size_t rows = n, cols = std::strtoull(argv[3], nullptr, 10);
    std::vector<T> a = read_file<T>(argv[4], rows * cols);
    nt2::table<T> A(nt2::of_size(rows, cols)), At(nt2::of_size(cols, rows)), C(nt2::of_size(5, 7)), B;
    load(A, a);
    load(At, a);
    for (std::size_t i = 1; i <= 35; ++i) C(i) = T(i);
    B = A * T(2) + T(1);
    std::printf("B1 %zu %zu\n", B.height(), B.width());
    write_table(argv[5], B);
    B = At + T(1);
    std::printf("B2 %zu %zu\n", B.height(), B.width());
    write_table(argv[6], B);
    B = C * T(3);
    std::printf("B3 %zu %zu\n", B.height(), B.width());
    write_table(argv[7], B);
    const T g1 = nt2::globalsum(C), g2 = nt2::globalsum(C * C);
    std::printf("G %.9g %.9g\n", (double)g1, (double)g2);
  } else {
    std::fprintf(stderr, "unknown demo %s\n", cmd.c_str());
    return 2;
  }
  return 0;
}
