// hpxfft::shared::opt -- drop-in for core/include/hpxfft/shared/opt.hpp.
// The reference's task variants differ only in HPX synchronisation; on the
// GPU the transform is one stream-ordered pair of kernels.
#pragma once
#ifndef hpxfft_shared_opt_H_INCLUDED
#define hpxfft_shared_opt_H_INCLUDED

#include <string>

#include "../util/gpu_plan.hpp"
#include "../util/vector_2d.hpp"

typedef double real;

namespace hpxfft::shared
{
using vector_2d = hpxfft::util::vector_2d<real>;

struct opt
{
  public:
    opt() = default;

    void initialize(vector_2d values_vec, const std::string PLAN_FLAG)
    {
        impl_.initialize_impl(std::move(values_vec), PLAN_FLAG);
    }

    vector_2d fft_2d_r2c() { return impl_.run(); }

    real get_measurement(std::string name) { return impl_.measurement(name); }

  private:
    hpxfft::util::gpu_transform<real> impl_;
};
}  // namespace hpxfft::shared
#endif
