// Shared machinery of the drop-in classes: a plan over the C ABI, the
// move-in / move-out ownership of the reference's classes and its
// measurement map.  Status codes of the C ABI become the reference's
// exception types: HPXFFT_ERR_INVALID_ARG -> std::invalid_argument (as
// string_to_fftw_plan_flag throws, core/include/hpxfft/util/adapter_fftw.hpp:42),
// HPXFFT_ERR_IO -> std::runtime_error (core/src/shared/loop.cpp:197-201),
// anything else -> std::runtime_error.
#pragma once
#include <map>
#include <stdexcept>
#include <string>

#include "../../../../include/hpxfft_gb300.h"
#include "vector_2d.hpp"

namespace hpxfft::util {

inline void check_status(int status)
{
    if (status == HPXFFT_OK) return;
    std::string msg = std::string(hpxfft_status_string(status)) + ": " + hpxfft_last_error();
    if (status == HPXFFT_ERR_INVALID_ARG) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

// Plan flag validation with the reference's exception
// (core/include/hpxfft/util/adapter_fftw.hpp:22-44).
inline void validate_plan_flag(const std::string &flag)
{
    if (!hpxfft_plan_flag_valid(flag.c_str())) throw std::invalid_argument("Invalid FFTW plan flag string");
}

// Precision of the plan for element type T: FP64 (float-float) for double,
// FP32 for float; PREC overrides it (HPXFFT_PREC_BF16X3 for float buffers,
// HPXFFT_PREC_F64_NATIVE for double ones).
template <typename T>
constexpr int default_precision()
{
    return sizeof(T) == 4 ? HPXFFT_PREC_F32 : HPXFFT_PREC_F64;
}

template <typename T, int PREC = default_precision<T>()>
class gpu_transform {
  public:
    using vector_type = vector_2d<T>;

    gpu_transform() = default;
    gpu_transform(const gpu_transform &) = delete;
    gpu_transform &operator=(const gpu_transform &) = delete;
    ~gpu_transform() { reset(); }

    // initialize(values, PLAN_FLAG): moves the data in and plans
    // (core/src/shared/loop.cpp:158-189).
    void initialize_impl(vector_type values_vec, const std::string &plan_flag)
    {
        validate_plan_flag(plan_flag);
        reset();
        static_assert((sizeof(T) == 4) == (PREC == HPXFFT_PREC_F32 || PREC == HPXFFT_PREC_BF16X3),
                      "float buffers need an FP32-storage precision, double buffers an FP64 one");
        check_status(hpxfft_plan_create(&plan_, values_vec.n_row(), values_vec.n_col(), 1, PREC, plan_flag.c_str()));
        n_row_ = values_vec.n_row();
        n_col_ = values_vec.n_col();
        values_ = std::move(values_vec);
        for (const char *k : {"plan", "plan_flops"}) {
            double v = 0.0;
            hpxfft_get_measurement(plan_, k, &v);
            measurements_[k] = v;
        }
    }

    // the transform; the result is moved out (core/src/shared/loop.cpp:112)
    vector_type run()
    {
        if (!plan_) throw std::runtime_error("initialize() must be called before the transform");
        check_status(hpxfft_execute_r2c_host(plan_, values_.data()));
        read_measurements();
        return std::move(values_);
    }

    // gradient of a loss of the spectrum: grad holds dL/dRe X + i dL/dIm X in
    // the output layout; returns dL/dx in the input layout (pads 0).  The
    // plan stays usable; no reference counterpart.
    vector_type run_backward(vector_type grad)
    {
        if (!plan_) throw std::runtime_error("initialize() must be called before the transform");
        if (grad.n_row() != n_row_ || grad.n_col() != n_col_)
            throw std::invalid_argument("gradient must have the planned n_row x n_col layout");
        check_status(hpxfft_execute_r2c_backward_host(plan_, grad.data()));
        read_measurements();
        return grad;
    }

    double measurement(const std::string &name) { return measurements_[name]; }

    void write_plans(const std::string &file_path)
    {
        if (!plan_) throw std::runtime_error("initialize() must be called before write_plans_to_file");
        const int rc = hpxfft_write_plan(plan_, file_path.c_str());
        if (rc == HPXFFT_ERR_IO) throw std::runtime_error("Failed to open file: " + file_path);
        check_status(rc);
    }

    std::map<std::string, double> &measurements() { return measurements_; }

  private:
    void read_measurements()
    {
        for (const char *k : {"total", "first_fftw", "first_trans", "second_fftw", "second_trans", "h2d", "d2h", "e2e",
                              "gbps", "gflops", "roofline"}) {
            double v = 0.0;
            hpxfft_get_measurement(plan_, k, &v);
            measurements_[k] = v;
        }
    }
    void reset()
    {
        if (plan_) hpxfft_plan_destroy(plan_);
        plan_ = nullptr;
    }
    hpxfft_plan plan_ = nullptr;
    std::size_t n_row_ = 0, n_col_ = 0;
    vector_type values_;
    std::map<std::string, double> measurements_;
};

}  // namespace hpxfft::util
