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

struct loop
{
  public:
    loop() = default;

    void initialize(vector_2d values_vec, const std::string PLAN_FLAG)
    {
        impl_.initialize_impl(std::move(values_vec), PLAN_FLAG);
    }

    vector_2d fft_2d_r2c_par() { return impl_.run(); }

    // the reference's seq variant overruns its transpose when nx > ny/2+1
    // (core/src/shared/loop.cpp:126-130); here it is the same transform
    vector_2d fft_2d_r2c_seq() { return impl_.run(); }

    vector_2d fft_2d_r2c() { return impl_.run(); }

    real get_measurement(std::string name) { return impl_.measurement(name); }

    void write_plans_to_file(std::string file_path) { impl_.write_plans(file_path); }

  private:
    hpxfft::util::gpu_transform<real> impl_;
};
}  // namespace hpxfft::shared
#endif  // hpxfft_shared_loop_H_INCLUDED
