/*
 * Stand-in for the cv::Mat / cv::imread subset that the reference's CPU
 * DPRA uses (DPRA/dpra_cpu.h, DPRA/dpra_cpu.cpp: an 8-bit single-channel
 * frame read with at<uchar>(row, col)), so that the file compiles here as it
 * is.  TEST INFRASTRUCTURE ONLY (oracle/ref_build.py installs it as
 * opencv2/opencv.hpp under oracle/_ref).  imread is not supported: frames
 * come from memory.
 */
#ifndef GLSU_REF_OPENCV_SHIM_HPP
#define GLSU_REF_OPENCV_SHIM_HPP

#include <cstddef>
#include <memory>
#include <string>
#include <vector>

typedef unsigned char uchar;

namespace cv {

class Mat {
public:
    int rows = 0, cols = 0;
    Mat() {}
    Mat(int r, int c) : rows(r), cols(c), buf_(std::make_shared<std::vector<uchar>>((size_t)r * c)) {}
    template <typename T> T &at(int r, int c) { return reinterpret_cast<T *>(buf_->data())[(size_t)r * cols + c]; }
    template <typename T> const T &at(int r, int c) const
    {
        return reinterpret_cast<const T *>(buf_->data())[(size_t)r * cols + c];
    }
    uchar *data() { return buf_ ? buf_->data() : nullptr; }
    void reserve(size_t) {}
    bool empty() const { return !buf_ || buf_->empty(); }

private:
    std::shared_ptr<std::vector<uchar>> buf_;
};

inline Mat imread(const std::string &) { return Mat(); }

}  // namespace cv

#endif
