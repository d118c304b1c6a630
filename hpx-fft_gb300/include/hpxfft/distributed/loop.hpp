// hpxfft::distributed::loop -- drop-in for
// core/include/hpxfft/distributed/loop.hpp:17-31 at one locality.  The
// reference's scatter / all_to_all exchange (core/src/distributed/loop.cpp:39-84)
// is the identity at one locality; the per-locality compute is the same GPU
// transform as hpxfft::shared::loop.  An unknown COMM_FLAG throws
// std::invalid_argument (the reference prints and finalizes,
// core/src/distributed/loop.cpp:342-346).
#pragma once
#ifndef hpxfft_distributed_loop_H_INCLUDED
#define hpxfft_distributed_loop_H_INCLUDED

#include <stdexcept>
#include <string>

#include "../util/gpu_plan.hpp"
#include "../util/vector_2d.hpp"

typedef double real;

namespace hpxfft::distributed
{
using vector_2d = hpxfft::util::vector_2d<real>;

struct loop
{
  public:
    loop() = default;

    void initialize(vector_2d values_vec, const std::string COMM_FLAG, const std::string PLAN_FLAG)
    {
        if (COMM_FLAG != "scatter" && COMM_FLAG != "all_to_all")
            throw std::invalid_argument("Specify communication scheme: scatter or all_to_all");
        impl_.initialize_impl(std::move(values_vec), PLAN_FLAG);
    }

    vector_2d fft_2d_r2c()
    {
        vector_2d out = impl_.run();
        for (const char *k : {"first_split", "first_comm", "second_split", "second_comm"})
            impl_.measurements()[k] = 0.0;
        return out;
    }

    real get_measurement(std::string name) { return impl_.measurement(name); }

  private:
    hpxfft::util::gpu_transform<real> impl_;
};
}  // namespace hpxfft::distributed
#endif
