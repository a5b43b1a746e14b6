// glsu_classes.hpp -- the reference's C++ class interfaces, backed by the C ABI.
//
// Drop-in replacements (paths inside the reference project):
//   WFT_FPA::WFT::WFT2_CUDAF / WFT2_CUDA      WFT/WFT2_CUDAf.h:11-40, WFT/WFT2_CUDA.h:11-40
//   WFT_FPA::WFT::WFT2_DeviceResults[F]        WFT/WFT.h:92-135 (owns m_d_filtered and the WFR maps)
//   DPRA::DPRA_CUDAF                            DPRA/dpra_cudaf.h:21-46
//   DPRA::DPRA_CUDA  (empty in the reference)   DPRA/dpra_cuda.h:9-14; interface of DPRA_CPU, dpra_cpu.h:30-64
//   DPRA::DPRA_HYBRIDF / DPRA_HYBRID            DPRA/dpra_hybridf.h:15-40, DPRA/dpra_hybrid.h:15-40
//   AIA::AIA_CUDAF                              AIA/aia_cudaf.h:15-38
// Aliases WFF2_CUDAF / WFF2_CUDA name the WFF-only use.
//
// Differences from the reference, all deliberate:
//   - failures throw std::runtime_error (the reference calls exit() or
//     throws int -1); the C ABI underneath returns status codes;
//   - the per-parameter WFT2 constructor sets the y lower bound from wyl (the
//     reference assigns m_rWyl(rWxl), WFT/WFT2_CUDAf.cu:903);
//   - WFT_TYPE::WFR follows the CPU reference's formulation (truncated
//     window, WFT/WFT2_CPU.cpp:391-694), as WFF does;
//   - DPRA_CUDAF's batch operator() overloads, empty in the reference
//     (DPRA/dpra_cudaf.cu:193-205), run the DPRA_CPU::operator() loop;
//   - times are in milliseconds everywhere.
// Without OpenCV a minimal cv::Mat / cv::imread (8-bit and 24-bit BMP)
// stands in; define GLSU_HAVE_OPENCV to use the real one.
#pragma once

#include <cuComplex.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "glsu.h"

#ifdef GLSU_HAVE_OPENCV
#include <opencv2/opencv.hpp>
#else
namespace cv {
constexpr int CV_8UC1 = 0;
constexpr int CV_32FC1 = 5;
// Minimal single-channel image: rows x cols, row-major, owning its pixels.
class Mat {
  public:
    int rows = 0, cols = 0;
    int type_ = CV_8UC1;
    unsigned char *data = nullptr;
    Mat() = default;
    Mat(int r, int c, int t) : rows(r), cols(c), type_(t), buf_((size_t)r * c * (t == CV_32FC1 ? 4 : 1))
    {
        data = buf_.data();
    }
    Mat(const Mat &o) : rows(o.rows), cols(o.cols), type_(o.type_), buf_(o.buf_) { data = buf_.data(); }
    Mat &operator=(const Mat &o)
    {
        rows = o.rows; cols = o.cols; type_ = o.type_; buf_ = o.buf_; data = buf_.data();
        return *this;
    }
    int type() const { return type_; }
    bool empty() const { return buf_.empty(); }
    template <typename T> T &at(int y, int x) { return reinterpret_cast<T *>(data)[(size_t)y * cols + x]; }
    template <typename T> const T &at(int y, int x) const
    {
        return reinterpret_cast<const T *>(data)[(size_t)y * cols + x];
    }
    void reserve(int) {}

  private:
    std::vector<unsigned char> buf_;
};
// 8-bit grey (paletted) or 24-bit BMP -> CV_8UC1, top-down, grey as OpenCV's BGR2GRAY.
Mat imread(const std::string &path);
namespace cuda {
using HostMem = Mat;
}
}  // namespace cv
#endif

namespace WFT_FPA {
namespace WFT {

enum class WFT_TYPE { WFF, WFR };

// H*W device arrays allocated by the WFT2 constructor: m_d_filtered for
// WFT_TYPE::WFF, the eight ridge maps for WFT_TYPE::WFR.
struct WFT2_DeviceResultsF {
    cuFloatComplex *m_d_filtered = nullptr;
    float *m_d_wx = nullptr;          // local frequency in x
    float *m_d_wy = nullptr;          // local frequency in y
    float *m_d_phase = nullptr;       // phase
    float *m_d_phase_comp = nullptr;  // compensated by the estimation of c
    float *m_d_b = nullptr;           // amplitude
    float *m_d_r = nullptr;           // ridge value
    float *m_d_cxx = nullptr;         // estimation of c in x
    float *m_d_cyy = nullptr;         // estimation of c in y
    WFT2_DeviceResultsF() = default;
    WFT2_DeviceResultsF(const WFT2_DeviceResultsF &) = delete;
    ~WFT2_DeviceResultsF();
};

struct WFT2_DeviceResults {
    cuDoubleComplex *m_d_filtered = nullptr;
    double *m_d_wx = nullptr, *m_d_wy = nullptr, *m_d_phase = nullptr, *m_d_phase_comp = nullptr;
    double *m_d_b = nullptr, *m_d_r = nullptr, *m_d_cxx = nullptr, *m_d_cyy = nullptr;
    WFT2_DeviceResults() = default;
    WFT2_DeviceResults(const WFT2_DeviceResults &) = delete;
    ~WFT2_DeviceResults();
};

class WFT2_CUDAF {
  public:
    WFT2_CUDAF() = delete;
    WFT2_CUDAF(const WFT2_CUDAF &) = delete;
    WFT2_CUDAF &operator=(const WFT2_CUDAF &) = delete;
    // Default parameters of the WFT_TYPE (WFT/WFT2_CUDAf.cu:852-875)
    WFT2_CUDAF(int iWidth, int iHeight, WFT_TYPE type, WFT2_DeviceResultsF &z, int iNumStreams = 1);
    WFT2_CUDAF(int iWidth, int iHeight, WFT_TYPE type, float rSigmaX, float rWxl, float rWxh, float rWxi,
               float rSigmaY, float rWyl, float rWyh, float rWyi, float rThr, WFT2_DeviceResultsF &z,
               int iNumStreams = 1);
    ~WFT2_CUDAF();
    // d_f: device W*H input; d_z.m_d_filtered (WFF) or the ridge maps (WFR)
    // receive the result; time in ms
    void operator()(cuFloatComplex *d_f, WFT2_DeviceResultsF &d_z, double &time);
    glsu_wff *handle() const { return h_; }
    glsu_wfr *wfr_handle() const { return hr_; }

  private:
    glsu_wff *h_ = nullptr;
    glsu_wfr *hr_ = nullptr;
    int w_, hgt_;
};

class WFT2_CUDA {
  public:
    WFT2_CUDA() = delete;
    WFT2_CUDA(const WFT2_CUDA &) = delete;
    WFT2_CUDA &operator=(const WFT2_CUDA &) = delete;
    WFT2_CUDA(int iWidth, int iHeight, WFT_TYPE type, WFT2_DeviceResults &z, int iNumStreams = 1);
    WFT2_CUDA(int iWidth, int iHeight, WFT_TYPE type, double rSigmaX, double rWxl, double rWxh, double rWxi,
              double rSigmaY, double rWyl, double rWyh, double rWyi, double rThr, WFT2_DeviceResults &z,
              int iNumStreams = 1);
    ~WFT2_CUDA();
    void operator()(cuDoubleComplex *d_f, WFT2_DeviceResults &d_z, double &time);
    glsu_wff *handle() const { return h_; }
    glsu_wfr *wfr_handle() const { return hr_; }

  private:
    glsu_wff *h_ = nullptr;
    glsu_wfr *hr_ = nullptr;
    int w_, hgt_;
};

using WFF2_CUDAF = WFT2_CUDAF;
using WFF2_CUDA = WFT2_CUDA;

}  // namespace WFT
}  // namespace WFT_FPA

namespace DPRA {

class DPRA_CUDAF {
  public:
    DPRA_CUDAF() = delete;
    DPRA_CUDAF(const DPRA_CUDAF &) = delete;
    DPRA_CUDAF &operator=(const DPRA_CUDAF &) = delete;
    // Phi0: HOST pointer, W*H row-major (DPRA/dpra_cudaf.h:28-30); the reference's
    // hard-wired 3x3 window and WFF parameters (DPRA/dpra_cudaf.cu:116-118).
    DPRA_CUDAF(const float *Phi0, const int iWidth, const int iHeight, const int irefUpdateRate = 1);
    // Window radius r ((2r+1)^2 window) and WFF parameters (sigma, low, high, step, thr).
    DPRA_CUDAF(const float *Phi0, const int iWidth, const int iHeight, const int irefUpdateRate, int iWindowRadius,
               const glsu_wff_params &wff);
    ~DPRA_CUDAF();

    void operator()(const std::vector<cv::cuda::HostMem> &f, std::vector<std::vector<float>> &dPhi_Sum,
                    double &time);
    void operator()(const std::vector<std::string> &fileNames, std::vector<std::vector<float>> &dPhi_Sum,
                    double &time);
    // img: CV_8UC1 (or CV_32FC1) H x W; dPhi resized to W*H if empty
    void dpra_per_frame(const cv::Mat &img, std::vector<float> &dPhi, double &time);
    void update_ref_phi();
    // Current (wrapped) phase, which the reference does not expose.
    void get_phi_curr(std::vector<float> &phi) const;
    glsu_dpra *handle() const { return h_; }
    int ref_update_rate() const { return rr_; }

  private:
    glsu_dpra *h_ = nullptr;
    int w_, hgt_, rr_;
};

class DPRA_CUDA {
  public:
    DPRA_CUDA() = delete;
    DPRA_CUDA(const DPRA_CUDA &) = delete;
    DPRA_CUDA &operator=(const DPRA_CUDA &) = delete;
    DPRA_CUDA(const double *v_Phi0, const int iWidth, const int iHeight, const int irefUpdateRate = 1);
    DPRA_CUDA(const double *v_Phi0, const int iWidth, const int iHeight, const int irefUpdateRate,
              int iWindowRadius, const glsu_wff_params &wff);
    ~DPRA_CUDA();
    void operator()(const std::vector<cv::Mat> &f, std::vector<std::vector<double>> &dPhi_Sum, double &time);
    void operator()(const std::vector<std::string> &fileNames, std::vector<std::vector<double>> &dPhi_Sum,
                    double &time);
    void dpra_per_frame(const cv::Mat &f, std::vector<double> &dPhi, double &time);
    void update_ref_phi();
    void get_phi_curr(std::vector<double> &phi) const;
    glsu_dpra *handle() const { return h_; }

  private:
    glsu_dpra *h_ = nullptr;
    int w_, hgt_, rr_;
};

// DPRA::DPRA_HYBRIDF / DPRA_HYBRID (DPRA/dpra_hybridf.h:15-40,
// DPRA/dpra_hybrid.h:15-40).  The reference builds the window sums on the GPU,
// copies them to the host, solves the 3x3 systems there with LAPACKE_dsysv on
// iNumThreads OpenMP threads and filters on the GPU again
// (DPRA/dpra_hybrid.cpp:182-270).  Here the whole frame stays on the GPU: the
// classes are the DPRA_CUDAF / DPRA_CUDA path with the same hard-wired 3x3
// window and WFF parameters (DPRA/dpra_hybrid.cpp:34-36), so iNumThreads is
// accepted and unused and the results equal those classes' bit for bit.
class DPRA_HYBRIDF : public DPRA_CUDAF {
  public:
    DPRA_HYBRIDF() = delete;
    DPRA_HYBRIDF(const DPRA_HYBRIDF &) = delete;
    DPRA_HYBRIDF &operator=(const DPRA_HYBRIDF &) = delete;
    DPRA_HYBRIDF(const float *v_Phi0, const int iWidth, const int iHeight, const int irefUpdateRate = 1,
                 const int iNumThreads = 1)
        : DPRA_CUDAF(v_Phi0, iWidth, iHeight, irefUpdateRate)
    {
        (void)iNumThreads;
    }
    using DPRA_CUDAF::operator();
    // frames as cv::Mat (DPRA_CUDAF's takes cv::cuda::HostMem); DPRA_CPU::operator() loop
    void operator()(const std::vector<cv::Mat> &f, std::vector<std::vector<float>> &dPhi_Sum, double &time)
    {
        time = 0;
        std::vector<float> d;
        for (size_t i = 0; i < f.size(); i++) {
            double t = 0;
            dpra_per_frame(f[i], d, t);
            time += t;
            dPhi_Sum.push_back(d);
            if (i % ref_update_rate() == 0) update_ref_phi();
        }
    }
};

class DPRA_HYBRID : public DPRA_CUDA {
  public:
    DPRA_HYBRID() = delete;
    DPRA_HYBRID(const DPRA_HYBRID &) = delete;
    DPRA_HYBRID &operator=(const DPRA_HYBRID &) = delete;
    DPRA_HYBRID(const double *v_Phi0, const int iWidth, const int iHeight, const int irefUpdateRate = 1,
                const int iNumThreads = 1)
        : DPRA_CUDA(v_Phi0, iWidth, iHeight, irefUpdateRate)
    {
        (void)iNumThreads;
    }
};

}  // namespace DPRA

namespace AIA {

class AIA_CUDAF {
  public:
    AIA_CUDAF() = delete;
    AIA_CUDAF(const AIA_CUDAF &) = delete;
    AIA_CUDAF &operator=(const AIA_CUDAF &) = delete;
    explicit AIA_CUDAF(const std::vector<cv::Mat> &v_f);
    AIA_CUDAF(const int iM, const int icols, const int irows);
    ~AIA_CUDAF();
    // v_deltas: in/out; drawn from N(0,1) with d[0]=0 when its size != M
    // (seeded by the seed argument instead of the clock).
    void operator()(std::vector<float> &v_phi, std::vector<float> &v_deltas, double &runningtime, int &iters,
                    float &err, const std::vector<cv::Mat> &v_f, int iMaxIterations = 20, float dMaxErr = 1e-4f,
                    int iNumThreads = 1, uint64_t seed = 0);

  private:
    glsu_aia *h_ = nullptr;
    int M_, cols_, rows_;
};

}  // namespace AIA
