// Host-only checks of the drop-in C++ classes: everything they decide before
// a plan touches the device, so it runs on a machine without a GPU.  The
// exception types are the reference's: a bad plan flag throws
// std::invalid_argument (core/include/hpxfft/util/adapter_fftw.hpp:42),
// vector_2d::at out of range and a file that cannot be opened throw
// std::runtime_error (core/include/hpxfft/util/vector_2d.hpp:218-221,
// core/src/shared/loop.cpp:197-201), and get_measurement of an unknown key
// returns 0 (core/src/shared/loop.cpp:192).  Exit status 0 when every check
// passes.
#include <cstdio>
#include <stdexcept>
#include <string>
#include <utility>

#include "hpxfft/distributed/loop.hpp"
#include "hpxfft/shared/loop.hpp"
#include "hpxfft/shared/naive.hpp"
#include "hpxfft/shared/opt.hpp"
#include "hpxfft/shared/sync.hpp"

static int failures = 0;
#define REQUIRE(cond)                                                                   \
    do {                                                                                \
        if (!(cond)) {                                                                  \
            std::fprintf(stderr, "%s:%d: REQUIRE(%s) failed\n", __FILE__, __LINE__, #cond); \
            ++failures;                                                                 \
        }                                                                               \
    } while (0)

template <class E, class F>
static bool throws(F &&f)
{
    try {
        f();
    } catch (const E &) {
        return true;
    } catch (...) {
        return false;
    }
    return false;
}

template <class T>
static hpxfft::util::vector_2d<T> fixture(std::size_t n_col = 6)
{
    hpxfft::util::vector_2d<T> v(4, n_col, T(0));
    for (std::size_t i = 0; i < 4; ++i)
        for (std::size_t j = 0; j < 4; ++j) v(i, j) = T(j + 1);
    return v;
}

// the reference's classes with fft_2d_r2c(): a bad plan flag, a transform
// before initialize, an unknown measurement key
template <class F>
static void plan_errors()
{
    {
        F f;
        REQUIRE(throws<std::invalid_argument>([&] { f.initialize(fixture<double>(), "fastest"); }));
    }
    {
        F f;
        REQUIRE(throws<std::runtime_error>([&] { f.fft_2d_r2c(); }));
        REQUIRE(f.get_measurement("no_such_key") == 0.0);
    }
}

int main()
{
    // vector_2d (test/src/test_vector_2d.cpp:6-33), plus the ownership the
    // reference gets wrong: copies copy, moves empty the source
    {
        hpxfft::util::vector_2d<double> v(3, 3, 4.0);
        REQUIRE(v.n_row() == 3 && v.n_col() == 3 && v.size() == 9 && v(2, 2) == 4.0);
        REQUIRE(throws<std::runtime_error>([&] { v.at(3, 0); }));
        REQUIRE(throws<std::runtime_error>([&] { v.at(2, 3); }));
        // like the reference, at() bounds the flat index i * n_col + j only:
        // (0, 3) is element 3, i.e. (1, 0)
        v(1, 0) = 7.0;
        REQUIRE(v.at(0, 3) == 7.0 && v.at(2, 2) == 4.0);
        v(1, 0) = 4.0;
        hpxfft::util::vector_2d<double> c;
        c = v;
        REQUIRE(c == v && v.size() == 9);
        c(0, 0) = 1.0;
        REQUIRE(!(c == v) && v(0, 0) == 4.0);
        hpxfft::util::vector_2d<double> m(std::move(c));
        REQUIRE(m.size() == 9 && m(0, 0) == 1.0 && c.size() == 0);
        hpxfft::util::vector_2d<float> f(2, 6, 1.5f);
        REQUIRE(f.size() == 12 && f(1, 5) == 1.5f);
    }
    plan_errors<hpxfft::shared::loop>();
    plan_errors<hpxfft::shared::naive>();
    plan_errors<hpxfft::shared::sync>();
    plan_errors<hpxfft::shared::opt>();
    {
        hpxfft::shared::loop f;
        REQUIRE(throws<std::runtime_error>([&] { f.fft_2d_r2c_par(); }));
        REQUIRE(throws<std::runtime_error>([&] { f.fft_2d_r2c_seq(); }));
        REQUIRE(throws<std::runtime_error>([&] { f.write_plans_to_file("plan.txt"); }));
        REQUIRE(throws<std::runtime_error>([&] { f.fft_2d_r2c_backward(fixture<double>()); }));
        // odd n_col: ny must be even (core/src/shared/loop.cpp:164-165)
        REQUIRE(throws<std::runtime_error>([&] { f.initialize(fixture<double>(5), "estimate"); }));
        REQUIRE(throws<std::runtime_error>([&] { f.fft_2d_r2c(); }));  // still not planned
    }
    {
        hpxfft::shared::loop_f32 f;
        REQUIRE(throws<std::invalid_argument>([&] { f.initialize(fixture<float>(), "Estimate"); }));
        hpxfft::shared::loop_bf16x3 b;
        REQUIRE(throws<std::invalid_argument>([&] { b.initialize(fixture<float>(), ""); }));
    }
    {
        hpxfft::distributed::loop f;
        REQUIRE(throws<std::invalid_argument>([&] { f.initialize(fixture<double>(), "broadcast", "estimate"); }));
        REQUIRE(throws<std::invalid_argument>([&] { f.initialize(fixture<double>(), "scatter", "fastest"); }));
        REQUIRE(throws<std::runtime_error>([&] { f.fft_2d_r2c(); }));
        REQUIRE(f.get_measurement("no_such_key") == 0.0);
    }
    if (failures) {
        std::fprintf(stderr, "%d check(s) failed\n", failures);
        return 1;
    }
    std::printf("all host-side drop-in checks passed\n");
    return 0;
}
