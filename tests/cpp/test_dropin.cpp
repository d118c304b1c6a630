// The reference's C++ tests (test/src/test_*.cpp), compiled against the
// drop-in headers and libhpxfft_gb300.so instead of HPX + FFTW.  Each case
// is the 4 x 6 fixture with rows [1,2,3,4,pad,pad]: initialize(std::move(values),
// plan) -> transform -> REQUIRE(total >= 0) and REQUIRE(out == expected).
// Exit status 0 when every check passes.
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "hpxfft/distributed/loop.hpp"
#include "hpxfft/shared/loop.hpp"
#include "hpxfft/shared/naive.hpp"
#include "hpxfft/shared/opt.hpp"
#include "hpxfft/shared/sync.hpp"

static int failures = 0;
#define REQUIRE(cond)                                                          \
    do {                                                                       \
        if (!(cond)) {                                                         \
            std::fprintf(stderr, "%s:%d: REQUIRE(%s) failed\n", __FILE__, __LINE__, #cond); \
            ++failures;                                                        \
        }                                                                      \
    } while (0)

using hpxfft::shared::vector_2d;

static vector_2d input()
{
    vector_2d values_vec(4, 6, 0.0);
    for (std::size_t i = 0; i < 4; ++i) {
        values_vec(i, 0) = 1.0;
        values_vec(i, 1) = 2.0;
        values_vec(i, 2) = 3.0;
        values_vec(i, 3) = 4.0;
    }
    return values_vec;
}

static vector_2d expected()
{
    vector_2d e(4, 6, 0.0);
    e(0, 0) = 40.0;
    e(0, 2) = -8.0;
    e(0, 3) = 8.0;
    e(0, 4) = -8.0;
    return e;
}

template <class F>
static void shared_case(const char *plan)
{
    F fft;
    vector_2d values_vec = input();
    fft.initialize(std::move(values_vec), plan);
    REQUIRE(values_vec.size() == 0);
    vector_2d out = fft.fft_2d_r2c();
    REQUIRE(fft.get_measurement("total") >= 0.0);
    REQUIRE(out == expected());
}

int main()
{
    // test/src/test_vector_2d.cpp:6-33
    {
        hpxfft::util::vector_2d<double> vec(3, 3, 4.0);
        REQUIRE(vec.n_row() == 3 && vec.n_col() == 3 && vec(0, 0) == 4.0 && vec(2, 2) == 4.0 && vec.size() == 9);
        bool threw = false;
        try {
            vec.at(3, 3);
        } catch (const std::runtime_error &) {
            threw = true;
        }
        REQUIRE(threw);
        REQUIRE((hpxfft::util::vector_2d<double>(2, 2, 5.0) == hpxfft::util::vector_2d<double>(2, 2, 5.0)));
        REQUIRE(!(hpxfft::util::vector_2d<double>(2, 2, 5.0) == hpxfft::util::vector_2d<double>(2, 2, 6.0)));
        hpxfft::util::vector_2d<double> copy;
        copy = vec;  // copies (the reference swaps)
        REQUIRE(copy == vec && vec.size() == 9);
    }
    // test/src/test_shared_loop.cpp:10-61
    {
        hpxfft::shared::loop fft2;
        std::string plan_flag = "estimate";
        vector_2d values_vec = input();
        fft2.initialize(std::move(values_vec), plan_flag);
        vector_2d out2 = fft2.fft_2d_r2c_par();
        REQUIRE(fft2.get_measurement(std::string("total")) >= 0.0);
        REQUIRE(fft2.get_measurement(std::string("plan_flops")) > 0.0);
        REQUIRE(out2 == expected());
        hpxfft::shared::loop fft1;
        fft1.initialize(input(), plan_flag);
        REQUIRE(fft1.fft_2d_r2c_seq() == expected());
    }
    shared_case<hpxfft::shared::naive>("estimate");  // test/src/test_naive.cpp
    shared_case<hpxfft::shared::sync>("estimate");   // test/src/test_shared_sync.cpp
    shared_case<hpxfft::shared::opt>("estimate");    // test/src/test_shared_opt.cpp
    // test/src/test_distributed_loop.cpp:11-51 at one locality
    for (const char *comm : {"scatter", "all_to_all"}) {
        hpxfft::distributed::loop fft;
        fft.initialize(input(), comm, "estimate");
        vector_2d out = fft.fft_2d_r2c();
        REQUIRE(fft.get_measurement("total") >= 0.0);
        REQUIRE(out == expected());
    }
    // precision variants: FP32 on the fixture, split-BF16 on the ramp
    // x[i][j] = j (closed form), and the adjoint of an impulse at DC
    {
        hpxfft::shared::loop_f32 f;
        hpxfft::util::vector_2d<float> v(4, 6, 0.0f);
        for (std::size_t i = 0; i < 4; ++i)
            for (std::size_t j = 0; j < 4; ++j) v(i, j) = (float)(j + 1);
        f.initialize(std::move(v), "estimate");
        hpxfft::util::vector_2d<float> out = f.fft_2d_r2c();
        REQUIRE(out(0, 0) == 40.0f && out(0, 2) == -8.0f && out(0, 3) == 8.0f && out(0, 4) == -8.0f);
        REQUIRE(f.get_measurement("gbps") >= 0.0);
    }
    {
        const std::size_t nx = 1024, ny = 16, nc = 2 * (ny / 2 + 1);
        hpxfft::shared::loop_bf16x3 f;
        hpxfft::util::vector_2d<float> v(nx, nc, 0.0f);
        for (std::size_t i = 0; i < nx; ++i)
            for (std::size_t j = 0; j < ny; ++j) v(i, j) = (float)j;
        f.initialize(std::move(v), "estimate");
        hpxfft::util::vector_2d<float> out = f.fft_2d_r2c();
        double err = 0.0, norm = 0.0;
        const double pi = 3.14159265358979323846;
        for (std::size_t kx = 0; kx < nx; ++kx)
            for (std::size_t k = 0; k <= ny / 2; ++k) {
                double re = 0.0, im = 0.0;
                if (kx == 0 && k == 0) re = nx * ny * (ny - 1) / 2.0;
                if (kx == 0 && k > 0) {  // nx ny / (exp(-2 pi i k / ny) - 1)
                    const double c = std::cos(2 * pi * k / ny) - 1.0, s = -std::sin(2 * pi * k / ny);
                    const double d = c * c + s * s;
                    re = nx * ny * c / d;
                    im = -(double)nx * ny * s / d;
                }
                const double dr = out(kx, 2 * k) - re, di = out(kx, 2 * k + 1) - im;
                err += dr * dr + di * di;
                norm += re * re + im * im;
            }
        REQUIRE(std::sqrt(err / norm) <= 2e-6);
    }
    {
        hpxfft::shared::loop f;
        f.initialize(input(), "estimate");
        vector_2d g(4, 6, 0.0);
        g(0, 0) = 1.0;  // L = Re X[0][0] = sum of the inputs
        vector_2d grad = f.fft_2d_r2c_backward(std::move(g));
        bool ones = true;
        for (std::size_t i = 0; i < 4; ++i)
            for (std::size_t j = 0; j < 6; ++j) ones = ones && std::fabs(grad(i, j) - (j < 4 ? 1.0 : 0.0)) < 1e-14;
        REQUIRE(ones);
        REQUIRE(f.fft_2d_r2c() == expected());  // the plan stays usable
    }
    // error behaviour
    {
        bool threw = false;
        try {
            hpxfft::shared::loop f;
            f.initialize(input(), "fastest");
        } catch (const std::invalid_argument &) {
            threw = true;
        }
        REQUIRE(threw);
        threw = false;
        try {
            hpxfft::distributed::loop f;
            f.initialize(input(), "broadcast", "estimate");
        } catch (const std::invalid_argument &) {
            threw = true;
        }
        REQUIRE(threw);
        threw = false;
        try {
            hpxfft::shared::loop f;
            f.initialize(input(), "estimate");
            f.write_plans_to_file("/nonexistent-dir/plan.txt");
        } catch (const std::runtime_error &) {
            threw = true;
        }
        REQUIRE(threw);
    }
    if (failures) {
        std::fprintf(stderr, "%d check(s) failed\n", failures);
        return 1;
    }
    std::printf("all drop-in checks passed\n");
    return 0;
}
