// hpxfft::shared::loop -- drop-in for core/include/hpxfft/shared/loop.hpp:15-31.
// Same names and signatures; the transform runs on the GPU through the C ABI.
#pragma once
#ifndef hpxfft_shared_loop_H_INCLUDED
#define hpxfft_shared_loop_H_INCLUDED

#include <string>

#include "../util/gpu_plan.hpp"
#include "../util/vector_2d.hpp"

typedef double real;

namespace hpxfft::shared
{
using vector_2d = hpxfft::util::vector_2d<real>;

// The reference's class with the element type and the GPU precision as
// parameters; `loop` is the reference's double / FP64 one.
template <typename T, int PREC = hpxfft::util::default_precision<T>()>
struct basic_loop
{
  public:
    using vector_type = hpxfft::util::vector_2d<T>;

    basic_loop() = default;

    void initialize(vector_type values_vec, const std::string PLAN_FLAG)
    {
        impl_.initialize_impl(std::move(values_vec), PLAN_FLAG);
    }

    vector_type fft_2d_r2c_par() { return impl_.run(); }

    // the reference's seq variant overruns its transpose when nx > ny/2+1
    // (core/src/shared/loop.cpp:126-130); here it is the same transform
    vector_type fft_2d_r2c_seq() { return impl_.run(); }

    vector_type fft_2d_r2c() { return impl_.run(); }

    // adjoint of the transform (gradient of a loss of the spectrum)
    vector_type fft_2d_r2c_backward(vector_type grad) { return impl_.run_backward(std::move(grad)); }

    double get_measurement(std::string name) { return impl_.measurement(name); }

    void write_plans_to_file(std::string file_path) { impl_.write_plans(file_path); }

  private:
    hpxfft::util::gpu_transform<T, PREC> impl_;
};

using loop = basic_loop<real>;
using loop_f32 = basic_loop<float>;                        // FP32 storage and arithmetic
using loop_bf16x3 = basic_loop<float, HPXFFT_PREC_BF16X3>; // split-BF16 tensor-core stages
}  // namespace hpxfft::shared
#endif  // hpxfft_shared_loop_H_INCLUDED
