// hpxfft_gpu_shared_loop: the command-line driver of the reference's
// examples/hpxfft/shared_loop_2d.cpp on the GPU drop-in.  Same options
// (--nx --ny --plan --run --header --result, "--key=value" or "--key value"),
// same ramp input x[i][j] = j, same console report and the same
// semicolon-separated rows appended to runtimes/runtimes_hpx_shared_loop.txt
// and plans/plan_hpx_shared_loop.txt.  The n_threads column holds 1 (one GPU).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <map>
#include <string>

#include "hpxfft/shared/loop.hpp"

static std::map<std::string, std::string> parse(int argc, char **argv)
{
    std::map<std::string, std::string> o = {{"nx", "8"},   {"ny", "14"},    {"plan", "estimate"},
                                            {"run", "par"}, {"header", "0"}, {"result", "0"}};
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        if (a.rfind("--", 0) != 0) continue;
        a = a.substr(2);
        std::string key = a, val;
        const auto eq = a.find('=');
        if (eq != std::string::npos) {
            key = a.substr(0, eq);
            val = a.substr(eq + 1);
        } else if (i + 1 < argc) {
            val = argv[++i];
        }
        if (!o.count(key)) {
            std::cerr << "unknown option --" << key << "\n";
            std::exit(2);
        }
        o[key] = val;
    }
    return o;
}

static bool truthy(const std::string &s) { return s == "1" || s == "true" || s == "yes"; }

int main(int argc, char **argv)
{
    auto opt = parse(argc, argv);
    const std::string run_flag = opt["run"], plan_flag = opt["plan"];
    const bool print_result = truthy(opt["result"]), print_header = truthy(opt["header"]);
    const std::size_t dim_c_x = std::stoull(opt["nx"]);
    const std::size_t dim_r_y = std::stoull(opt["ny"]);
    const std::size_t dim_c_y = dim_r_y / 2 + 1;

    hpxfft::shared::vector_2d values_vec(dim_c_x, 2 * dim_c_y);
    for (std::size_t i = 0; i < dim_c_x; ++i)
        for (std::size_t j = 0; j < dim_r_y; ++j) values_vec(i, j) = (double)j;

    using clk = std::chrono::steady_clock;
    hpxfft::shared::loop fft_computer;
    const auto start_total = clk::now();
    fft_computer.initialize(std::move(values_vec), plan_flag);
    const auto stop_init = clk::now();
    values_vec = run_flag == "seq" ? fft_computer.fft_2d_r2c_seq() : fft_computer.fft_2d_r2c_par();
    const auto stop_total = clk::now();
    const double total = std::chrono::duration<double>(stop_total - start_total).count();
    const double init = std::chrono::duration<double>(stop_init - start_total).count();

    if (print_result) {
        for (std::size_t i = 0; i < values_vec.n_row(); ++i) {
            for (std::size_t j = 0; j < values_vec.n_col(); j += 2)
                std::printf("(%g,%g) ", values_vec(i, j), values_vec(i, j + 1));
            std::printf("\n");
        }
    }
    auto m = [&](const char *k) { return fft_computer.get_measurement(k); };
    std::cout << "\nLocality 0 - shared - " << run_flag << "\nTotal runtime : " << total
              << "\nInitialization: " << init << "\nFFT 2D runtime: " << m("total") << "\nFFTW r2c      : "
              << m("first_fftw") << "\nFirst trans   : " << m("first_trans") << "\nFFTW c2c      : "
              << m("second_fftw") << "\nSecond trans  : " << m("second_trans") << "\nPlan time     : " << m("plan")
              << "\nPlan flops    : " << m("plan_flops") << "\nHost to device: " << m("h2d")
              << "\nDevice to host: " << m("d2h") << std::endl;

    const std::string header = "n_threads;n_x;n_y;plan;run_flag;total;initialization;fft_2d_total;first_fftw;"
                               "first_trans;second_fftw;second_trans;plan_time;plan_flops;\n";
    auto row = [&]() {
        std::string r = "1;" + std::to_string(dim_c_x) + ";" + std::to_string(dim_r_y) + ";" + plan_flag + ";" +
                        run_flag + ";";
        for (double v : {total, init, m("total"), m("first_fftw"), m("first_trans"), m("second_fftw"),
                         m("second_trans"), m("plan"), m("plan_flops")})
            r += std::to_string(v) + ";";
        return r + "\n";
    };
    std::filesystem::create_directories("runtimes");
    std::ofstream runtime_file("runtimes/runtimes_hpx_shared_loop.txt", std::ios_base::app);
    if (print_header) runtime_file << header;
    runtime_file << row();
    runtime_file.close();
    std::filesystem::create_directories("plans");
    std::ofstream plan_info_file("plans/plan_hpx_shared_loop.txt", std::ios_base::app);
    plan_info_file << header << row();
    plan_info_file.close();
    fft_computer.write_plans_to_file("plans/plan_hpx_shared_loop.txt");
    return 0;
}
