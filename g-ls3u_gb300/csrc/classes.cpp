// classes.cpp -- the reference's C++ classes implemented on the C ABI.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>

#include "../../include/glsu_classes.hpp"

namespace {

void throw_if(int rc, const char *what)
{
    if (rc != GLSU_OK) throw std::runtime_error(std::string(what) + ": " + glsu_last_error());
}

glsu_wff_params make_params(double sx, double wxl, double wxh, double wxi, double sy, double wyl, double wyh,
                            double wyi, double thr)
{
    glsu_wff_params p;
    p.sigma_x = sx; p.wxl = wxl; p.wxh = wxh; p.wxi = wxi;
    p.sigma_y = sy; p.wyl = wyl; p.wyh = wyh; p.wyi = wyi;
    p.thr = thr;
    return p;
}

int img_type_of(const cv::Mat &m) { return m.type() == cv::CV_32FC1 ? GLSU_F32 : GLSU_U8; }

}  // namespace

#ifndef GLSU_HAVE_OPENCV
cv::Mat cv::imread(const std::string &path)
{
    std::ifstream in(path, std::ios::binary);
    std::vector<unsigned char> d((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    auto u32 = [&](size_t o) { return (uint32_t)d[o] | (uint32_t)d[o + 1] << 8 | (uint32_t)d[o + 2] << 16 | (uint32_t)d[o + 3] << 24; };
    auto u16 = [&](size_t o) { return (uint32_t)d[o] | (uint32_t)d[o + 1] << 8; };
    if (d.size() < 54 || d[0] != 'B' || d[1] != 'M') return Mat();
    const uint32_t off = u32(10), hdr = u32(14);
    const int32_t w = (int32_t)u32(18), h0 = (int32_t)u32(22);
    const uint32_t bpp = u16(28), comp = u32(30);
    if (comp != 0 || w <= 0) return Mat();
    const bool top_down = h0 < 0;
    const int h = top_down ? -h0 : h0;
    Mat m(h, w, CV_8UC1);
    auto grey = [](uint32_t r, uint32_t g, uint32_t b) {
        return (unsigned char)((r * 4899 + g * 9617 + b * 1868 + (1u << 13)) >> 14);
    };
    if (bpp == 8) {
        uint32_t ncol = u32(46);
        if (!ncol) ncol = 256;
        const size_t pal = 14 + hdr, stride = ((size_t)w + 3) & ~(size_t)3;
        for (int y = 0; y < h; y++) {
            const size_t row = off + stride * (size_t)(top_down ? y : h - 1 - y);
            for (int x = 0; x < w; x++) {
                const unsigned idx = d[row + x] < ncol ? d[row + x] : 0;
                m.at<unsigned char>(y, x) = grey(d[pal + 4 * idx + 2], d[pal + 4 * idx + 1], d[pal + 4 * idx]);
            }
        }
    } else if (bpp == 24) {
        const size_t stride = (3 * (size_t)w + 3) & ~(size_t)3;
        for (int y = 0; y < h; y++) {
            const size_t row = off + stride * (size_t)(top_down ? y : h - 1 - y);
            for (int x = 0; x < w; x++)
                m.at<unsigned char>(y, x) = grey(d[row + 3 * x + 2], d[row + 3 * x + 1], d[row + 3 * x]);
        }
    } else {
        return Mat();
    }
    return m;
}
#endif

namespace WFT_FPA {
namespace WFT {

template <typename Z> static void free_results(Z &z)
{
    void *ps[] = {z.m_d_filtered, z.m_d_wx, z.m_d_wy, z.m_d_phase, z.m_d_phase_comp,
                  z.m_d_b,        z.m_d_r,  z.m_d_cxx, z.m_d_cyy};
    for (void *p : ps)
        if (p) cudaFree(p);
    z.m_d_filtered = nullptr;
    z.m_d_wx = z.m_d_wy = z.m_d_phase = z.m_d_phase_comp = z.m_d_b = z.m_d_r = z.m_d_cxx = z.m_d_cyy = nullptr;
}

WFT2_DeviceResultsF::~WFT2_DeviceResultsF() { free_results(*this); }
WFT2_DeviceResults::~WFT2_DeviceResults() { free_results(*this); }

// Allocates the results of the WFT type: the filtered field for WFF, the
// eight ridge maps for WFR (element type E).
template <typename Z, typename C, typename E> static bool alloc_results(Z &z, WFT_TYPE type, size_t n)
{
    if (type == WFT_TYPE::WFF) return cudaMalloc((void **)&z.m_d_filtered, sizeof(C) * n) == cudaSuccess;
    E **maps[] = {&z.m_d_wx, &z.m_d_wy, &z.m_d_phase, &z.m_d_phase_comp, &z.m_d_b, &z.m_d_r, &z.m_d_cxx, &z.m_d_cyy};
    for (E **m : maps)
        if (cudaMalloc((void **)m, sizeof(E) * n) != cudaSuccess) return false;
    return true;
}

template <typename Z> static glsu_wfr_results wfr_maps(Z &z)
{
    glsu_wfr_results r;
    r.wx = z.m_d_wx;
    r.wy = z.m_d_wy;
    r.phase = z.m_d_phase;
    r.phase_comp = z.m_d_phase_comp;
    r.b = z.m_d_b;
    r.r = z.m_d_r;
    r.cxx = z.m_d_cxx;
    r.cyy = z.m_d_cyy;
    return r;
}

// Creates the handle of the WFT type (the other stays null).
static void make_wft(int prec, int w, int h, WFT_TYPE type, const glsu_wff_params *p, glsu_wff **hf,
                     glsu_wfr **hr)
{
    if (type == WFT_TYPE::WFF) throw_if(glsu_wff_create(hf, prec, w, h, p), "WFT2 construction failed");
    else throw_if(glsu_wfr_create(hr, prec, w, h, p), "WFT2 (WFR) construction failed");
}

static void destroy_wft(glsu_wff *hf, glsu_wfr *hr)
{
    glsu_wff_destroy(hf);
    glsu_wfr_destroy(hr);
}

WFT2_CUDAF::WFT2_CUDAF(int iWidth, int iHeight, WFT_TYPE type, WFT2_DeviceResultsF &z, int)
    : w_(iWidth), hgt_(iHeight)
{
    glsu_wff_params p;
    glsu_wft_default_params(type == WFT_TYPE::WFF ? GLSU_WFT_WFF : GLSU_WFT_WFR, &p);
    make_wft(GLSU_F32, iWidth, iHeight, type, &p, &h_, &hr_);
    if (!alloc_results<WFT2_DeviceResultsF, cuFloatComplex, float>(z, type, (size_t)iWidth * iHeight)) {
        destroy_wft(h_, hr_);
        throw std::runtime_error("cudaMalloc of the WFT2 results failed");
    }
}

WFT2_CUDAF::WFT2_CUDAF(int iWidth, int iHeight, WFT_TYPE type, float rSigmaX, float rWxl, float rWxh, float rWxi,
                       float rSigmaY, float rWyl, float rWyh, float rWyi, float rThr, WFT2_DeviceResultsF &z, int)
    : w_(iWidth), hgt_(iHeight)
{
    glsu_wff_params p = make_params(rSigmaX, rWxl, rWxh, rWxi, rSigmaY, rWyl, rWyh, rWyi, rThr);
    make_wft(GLSU_F32, iWidth, iHeight, type, &p, &h_, &hr_);
    if (!alloc_results<WFT2_DeviceResultsF, cuFloatComplex, float>(z, type, (size_t)iWidth * iHeight)) {
        destroy_wft(h_, hr_);
        throw std::runtime_error("cudaMalloc of the WFT2 results failed");
    }
}

WFT2_CUDAF::~WFT2_CUDAF() { destroy_wft(h_, hr_); }

void WFT2_CUDAF::operator()(cuFloatComplex *d_f, WFT2_DeviceResultsF &d_z, double &time)
{
    if (h_) {
        throw_if(glsu_wff_run(h_, d_f, d_z.m_d_filtered, &time), "WFF2 failed");
    } else {
        const glsu_wfr_results z = wfr_maps(d_z);
        throw_if(glsu_wfr_run(hr_, d_f, &z, &time), "WFR2 failed");
    }
}

WFT2_CUDA::WFT2_CUDA(int iWidth, int iHeight, WFT_TYPE type, WFT2_DeviceResults &z, int)
    : w_(iWidth), hgt_(iHeight)
{
    glsu_wff_params p;
    glsu_wft_default_params(type == WFT_TYPE::WFF ? GLSU_WFT_WFF : GLSU_WFT_WFR, &p);
    make_wft(GLSU_F64, iWidth, iHeight, type, &p, &h_, &hr_);
    if (!alloc_results<WFT2_DeviceResults, cuDoubleComplex, double>(z, type, (size_t)iWidth * iHeight)) {
        destroy_wft(h_, hr_);
        throw std::runtime_error("cudaMalloc of the WFT2 results failed");
    }
}

WFT2_CUDA::WFT2_CUDA(int iWidth, int iHeight, WFT_TYPE type, double rSigmaX, double rWxl, double rWxh, double rWxi,
                     double rSigmaY, double rWyl, double rWyh, double rWyi, double rThr, WFT2_DeviceResults &z, int)
    : w_(iWidth), hgt_(iHeight)
{
    glsu_wff_params p = make_params(rSigmaX, rWxl, rWxh, rWxi, rSigmaY, rWyl, rWyh, rWyi, rThr);
    make_wft(GLSU_F64, iWidth, iHeight, type, &p, &h_, &hr_);
    if (!alloc_results<WFT2_DeviceResults, cuDoubleComplex, double>(z, type, (size_t)iWidth * iHeight)) {
        destroy_wft(h_, hr_);
        throw std::runtime_error("cudaMalloc of the WFT2 results failed");
    }
}

WFT2_CUDA::~WFT2_CUDA() { destroy_wft(h_, hr_); }

void WFT2_CUDA::operator()(cuDoubleComplex *d_f, WFT2_DeviceResults &d_z, double &time)
{
    if (h_) {
        throw_if(glsu_wff_run(h_, d_f, d_z.m_d_filtered, &time), "WFF2 failed");
    } else {
        const glsu_wfr_results z = wfr_maps(d_z);
        throw_if(glsu_wfr_run(hr_, d_f, &z, &time), "WFR2 failed");
    }
}

}  // namespace WFT
}  // namespace WFT_FPA

namespace DPRA {

static glsu_dpra *make_dpra(int prec, const void *phi0, int w, int h, int rr, int r, const glsu_wff_params *p)
{
    glsu_dpra *hd = nullptr;
    throw_if(glsu_dpra_create(&hd, prec, phi0, w, h, rr, r, p), "DPRA construction failed");
    return hd;
}

DPRA_CUDAF::DPRA_CUDAF(const float *Phi0, const int iWidth, const int iHeight, const int irefUpdateRate)
    : w_(iWidth), hgt_(iHeight), rr_(irefUpdateRate)
{
    h_ = make_dpra(GLSU_F32, Phi0, iWidth, iHeight, irefUpdateRate, 1, nullptr);
}

DPRA_CUDAF::DPRA_CUDAF(const float *Phi0, const int iWidth, const int iHeight, const int irefUpdateRate,
                       int iWindowRadius, const glsu_wff_params &wff)
    : w_(iWidth), hgt_(iHeight), rr_(irefUpdateRate)
{
    h_ = make_dpra(GLSU_F32, Phi0, iWidth, iHeight, irefUpdateRate, iWindowRadius, &wff);
}

DPRA_CUDAF::~DPRA_CUDAF() { glsu_dpra_destroy(h_); }

void DPRA_CUDAF::dpra_per_frame(const cv::Mat &img, std::vector<float> &dPhi, double &time)
{
    if (img.cols != w_ || img.rows != hgt_)
        throw std::runtime_error("Size of the input FP is not equal to the size in the initialization");
    if (dPhi.size() != (size_t)w_ * hgt_) dPhi.resize((size_t)w_ * hgt_);
    throw_if(glsu_dpra_per_frame(h_, img.data, img_type_of(img), dPhi.data(), &time), "dpra_per_frame failed");
}

void DPRA_CUDAF::update_ref_phi() { throw_if(glsu_dpra_update_ref_phi(h_), "update_ref_phi failed"); }

void DPRA_CUDAF::get_phi_curr(std::vector<float> &phi) const
{
    phi.resize((size_t)w_ * hgt_);
    throw_if(glsu_dpra_get(h_, GLSU_PHI_CURR, phi.data()), "get_phi_curr failed");
}

void DPRA_CUDAF::operator()(const std::vector<cv::cuda::HostMem> &f, std::vector<std::vector<float>> &dPhi_Sum,
                            double &time)
{
    // DPRA_CPU::operator() semantics (DPRA/dpra_cpu.cpp:58-89)
    time = 0;
    std::vector<float> d((size_t)w_ * hgt_);
    for (size_t i = 0; i < f.size(); i++) {
        double t = 0;
        dpra_per_frame(f[i], d, t);
        time += t;
        dPhi_Sum.push_back(d);
        if (i % rr_ == 0) update_ref_phi();
    }
}

void DPRA_CUDAF::operator()(const std::vector<std::string> &fileNames, std::vector<std::vector<float>> &dPhi_Sum,
                            double &time)
{
    std::vector<cv::Mat> frames;
    for (const auto &n : fileNames) {
        frames.push_back(cv::imread(n));
        if (frames.back().empty()) throw std::runtime_error("cannot read " + n);
    }
    (*this)(frames, dPhi_Sum, time);
}

DPRA_CUDA::DPRA_CUDA(const double *v_Phi0, const int iWidth, const int iHeight, const int irefUpdateRate)
    : w_(iWidth), hgt_(iHeight), rr_(irefUpdateRate)
{
    h_ = make_dpra(GLSU_F64, v_Phi0, iWidth, iHeight, irefUpdateRate, 1, nullptr);
}

DPRA_CUDA::DPRA_CUDA(const double *v_Phi0, const int iWidth, const int iHeight, const int irefUpdateRate,
                     int iWindowRadius, const glsu_wff_params &wff)
    : w_(iWidth), hgt_(iHeight), rr_(irefUpdateRate)
{
    h_ = make_dpra(GLSU_F64, v_Phi0, iWidth, iHeight, irefUpdateRate, iWindowRadius, &wff);
}

DPRA_CUDA::~DPRA_CUDA() { glsu_dpra_destroy(h_); }

void DPRA_CUDA::dpra_per_frame(const cv::Mat &f, std::vector<double> &dPhi, double &time)
{
    if (f.cols != w_ || f.rows != hgt_)
        throw std::runtime_error("Size of the input FP is not equal to the size in the initialization");
    if (dPhi.size() != (size_t)w_ * hgt_) dPhi.resize((size_t)w_ * hgt_);
    throw_if(glsu_dpra_per_frame(h_, f.data, img_type_of(f), dPhi.data(), &time), "dpra_per_frame failed");
}

void DPRA_CUDA::update_ref_phi() { throw_if(glsu_dpra_update_ref_phi(h_), "update_ref_phi failed"); }

void DPRA_CUDA::get_phi_curr(std::vector<double> &phi) const
{
    phi.resize((size_t)w_ * hgt_);
    throw_if(glsu_dpra_get(h_, GLSU_PHI_CURR, phi.data()), "get_phi_curr failed");
}

void DPRA_CUDA::operator()(const std::vector<cv::Mat> &f, std::vector<std::vector<double>> &dPhi_Sum, double &time)
{
    time = 0;
    std::vector<double> d((size_t)w_ * hgt_);
    for (size_t i = 0; i < f.size(); i++) {
        double t = 0;
        dpra_per_frame(f[i], d, t);
        time += t;
        dPhi_Sum.push_back(d);
        if (i % rr_ == 0) update_ref_phi();
    }
}

void DPRA_CUDA::operator()(const std::vector<std::string> &fileNames, std::vector<std::vector<double>> &dPhi_Sum,
                           double &time)
{
    std::vector<cv::Mat> frames;
    for (const auto &n : fileNames) {
        frames.push_back(cv::imread(n));
        if (frames.back().empty()) throw std::runtime_error("cannot read " + n);
    }
    (*this)(frames, dPhi_Sum, time);
}

}  // namespace DPRA

namespace AIA {

AIA_CUDAF::AIA_CUDAF(const std::vector<cv::Mat> &v_f)
    : M_((int)v_f.size()), cols_(v_f.empty() ? 0 : v_f[0].cols), rows_(v_f.empty() ? 0 : v_f[0].rows)
{
    throw_if(glsu_aia_create(&h_, M_, cols_, rows_), "AIA construction failed");
}

AIA_CUDAF::AIA_CUDAF(const int iM, const int icols, const int irows) : M_(iM), cols_(icols), rows_(irows)
{
    throw_if(glsu_aia_create(&h_, iM, icols, irows), "AIA construction failed");
}

AIA_CUDAF::~AIA_CUDAF() { glsu_aia_destroy(h_); }

void AIA_CUDAF::operator()(std::vector<float> &v_phi, std::vector<float> &v_deltas, double &runningtime, int &iters,
                           float &err, const std::vector<cv::Mat> &v_f, int iMaxIterations, float dMaxErr, int,
                           uint64_t seed)
{
    if ((int)v_f.size() != M_) throw std::runtime_error("AIA: number of frames differs from construction");
    std::vector<const void *> ptrs;
    for (const auto &m : v_f) {
        if (m.cols != cols_ || m.rows != rows_) throw std::runtime_error("AIA: frame size mismatch");
        ptrs.push_back(m.data);
    }
    const int n_in = (int)v_deltas.size();
    v_deltas.resize(M_);
    v_phi.resize((size_t)cols_ * rows_);
    throw_if(glsu_aia_run(h_, ptrs.data(), img_type_of(v_f[0]), v_phi.data(), v_deltas.data(), n_in, &runningtime,
                          &iters, &err, iMaxIterations, dMaxErr, seed),
             "AIA failed");
}

}  // namespace AIA
