// hpxfft::util::vector_2d -- the reference's row-major 2D buffer
// (core/include/hpxfft/util/vector_2d.hpp:9-86), same interface.
//
// Differences, all deliberate:
//  - the buffer is freed by the destructor (the reference's never is,
//    vector_2d.hpp:31,104), copy assignment copies (the reference swaps,
//    :146-151) and the move constructor leaves the source empty;
//  - storage comes from pinned host memory when the GPU library can provide
//    it, so host<->device copies of the drop-in run at full link speed;
//    otherwise from the C++ heap;
//  - no HPX serialization (there is no remote action to pass it to).
#pragma once
#include <algorithm>
#include <cstddef>
#include <stdexcept>
#include <utility>

#include "../../../../include/hpxfft_gb300.h"

namespace hpxfft::util {

template <typename T>
struct vector_2d {
  public:
    using iterator = T *;
    using const_iterator = const T *;

    vector_2d() = default;
    vector_2d(std::size_t n_row, std::size_t n_col) : vector_2d(n_row, n_col, T()) {}
    vector_2d(std::size_t n_row, std::size_t n_col, const T &v) : n_row_(n_row), n_col_(n_col), size_(n_row * n_col)
    {
        allocate();
        std::fill(begin(), end(), v);
    }
    vector_2d(const vector_2d &src) : n_row_(src.n_row_), n_col_(src.n_col_), size_(src.size_)
    {
        allocate();
        std::copy(src.begin(), src.end(), begin());
    }
    vector_2d(vector_2d &&mv) noexcept { swap(*this, mv); }
    ~vector_2d() { release(); }

    vector_2d &operator=(const vector_2d &src)
    {
        if (this != &src) {
            vector_2d tmp(src);
            swap(*this, tmp);
        }
        return *this;
    }
    vector_2d &operator=(vector_2d &&mv) noexcept
    {
        if (this != &mv) {
            vector_2d tmp(std::move(mv));
            swap(*this, tmp);
        }
        return *this;
    }

    T &operator()(std::size_t i, std::size_t j) { return values_[i * n_col_ + j]; }
    const T &operator()(std::size_t i, std::size_t j) const { return values_[i * n_col_ + j]; }
    T &at(std::size_t i, std::size_t j)
    {
        if (i * n_col_ + j >= size_) throw std::runtime_error("out of range exception");
        return values_[i * n_col_ + j];
    }
    const T &at(std::size_t i, std::size_t j) const
    {
        if (i * n_col_ + j >= size_) throw std::runtime_error("out of range exception");
        return values_[i * n_col_ + j];
    }
    T *data() noexcept { return values_; }
    const T *data() const noexcept { return values_; }
    iterator begin() noexcept { return values_; }
    const_iterator begin() const noexcept { return values_; }
    iterator end() noexcept { return values_ + size_; }
    const_iterator end() const noexcept { return values_ + size_; }
    const_iterator cbegin() const noexcept { return values_; }
    const_iterator cend() const noexcept { return values_ + size_; }
    iterator row(std::size_t i) noexcept { return values_ + i * n_col_; }
    const_iterator row(std::size_t i) const noexcept { return values_ + i * n_col_; }
    std::size_t size() const noexcept { return size_; }
    std::size_t n_row() const noexcept { return n_row_; }
    std::size_t n_col() const noexcept { return n_col_; }

    template <typename H>
    friend bool operator==(const vector_2d<H> &lhs, const vector_2d<H> &rhs);

    friend void swap(vector_2d &a, vector_2d &b) noexcept
    {
        std::swap(a.values_, b.values_);
        std::swap(a.size_, b.size_);
        std::swap(a.n_row_, b.n_row_);
        std::swap(a.n_col_, b.n_col_);
        std::swap(a.pinned_, b.pinned_);
    }

  private:
    void allocate()
    {
        if (size_ == 0) return;
        void *p = nullptr;
        if (hpxfft_host_alloc(&p, size_ * sizeof(T)) == HPXFFT_OK && p) {
            values_ = static_cast<T *>(p);
            pinned_ = true;
        } else {
            values_ = new T[size_];
            pinned_ = false;
        }
    }
    void release() noexcept
    {
        if (!values_) return;
        if (pinned_)
            hpxfft_host_free(values_);
        else
            delete[] values_;
        values_ = nullptr;
    }

    T *values_ = nullptr;
    std::size_t n_row_ = 0, n_col_ = 0, size_ = 0;
    bool pinned_ = false;
};

template <typename H>
inline bool operator==(const vector_2d<H> &lhs, const vector_2d<H> &rhs)
{
    if (lhs.n_row_ != rhs.n_row_ || lhs.n_col_ != rhs.n_col_) return false;
    return std::equal(lhs.begin(), lhs.end(), rhs.begin());
}

}  // namespace hpxfft::util
