// ref_driver.cpp -- C entry points around the reference's own CPU classes
// (WFT_FPA::WFT::WFT2_cpu, WFT/WFT2_CPU.cpp; DPRA::DPRA_CPU,
// DPRA/dpra_cpu.cpp), compiled from the reference's sources by
// oracle/ref_build.py into oracle/_ref/libglsu_ref.so.  TEST INFRASTRUCTURE
// ONLY: it generates the golden vectors under tests/golden/ and is never
// part of the product.
//
// The DPRA class keeps its phases and its least-squares output private, so
// this translation unit (and only it) reads them by opening the class's
// access; the reference files are compiled unchanged.
#include <cstring>
#include <vector>

#define private public
#include "dpra_cpu.h"
#include "WFT2_CPU.h"
#undef private

using WFT_FPA::WFT::WFT2_cpu;
using WFT_FPA::WFT::WFT2_HostResults;
using WFT_FPA::WFT::WFT_TYPE;

extern "C" {

// WFF2 of an H x W complex field (interleaved re, im) with the reference's
// argument order (sigma, low, high, step for x, then y; thr < 0: automatic).
// out: H x W complex.  *thr_used receives the threshold the class used.
int ref_wff2(int W, int H, const double *p9, const double *f, double *out, double *thr_used, int nthreads)
{
    WFT2_HostResults z;
    WFT2_cpu wft(W, H, WFT_TYPE::WFF, p9[0], p9[1], p9[2], p9[3], p9[4], p9[5], p9[6], p9[7], p9[8], z,
                 nthreads);
    fftw_complex *in = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * (size_t)W * H);
    if (!in) return -1;
    std::memcpy(in, f, sizeof(double) * 2 * (size_t)W * H);
    double t = 0;
    wft(in, z, t);
    std::memcpy(out, z.m_filtered, sizeof(double) * 2 * (size_t)W * H);
    if (thr_used) *thr_used = wft.m_rThr;
    fftw_free(in);
    return 0;
}

// DPRA_CPU over a sequence of 8-bit frames (nframes x H x W), reference rate
// rr, with the reference's hard-wired 3x3 window and WFF parameters
// (DPRA/dpra_cpu.cpp:22-25), following DPRA_CPU::operator() (update after
// frame i when i % rr == 0).  Per frame: dphi (the returned phase change),
// phi_curr and the least-squares output exp(j dphi_ls) (complex); each
// output is nframes x H x W (complex: interleaved).
int ref_dpra_sequence(int W, int H, int nframes, const unsigned char *frames, const double *phi0, int rr,
                      int nthreads, double *dphi, double *phi_curr, double *lsq)
{
    DPRA::DPRA_CPU d(phi0, W, H, rr, nthreads);
    const size_t n = (size_t)W * H;
    std::vector<double> out(n, 0.0);
    for (int i = 0; i < nframes; i++) {
        cv::Mat m(H, W);
        std::memcpy(m.data(), frames + (size_t)i * n, n);
        double t = 0;
        d.dpra_per_frame(m, out, t);
        std::memcpy(dphi + (size_t)i * n, out.data(), sizeof(double) * n);
        std::memcpy(phi_curr + (size_t)i * n, d.m_PhiCurr.data(), sizeof(double) * n);
        std::memcpy(lsq + 2 * (size_t)i * n, d.m_dPhiWFT, sizeof(double) * 2 * n);
        if (i % rr == 0) d.update_ref_phi();
    }
    return 0;
}

}  // extern "C"
