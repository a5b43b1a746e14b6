// Driver for the C++ class tests: uses the reference's class names and
// signatures (DPRA_CUDAF, DPRA_CUDA, DPRA_HYBRID[F], WFT2_CUDAF, WFF2_CUDA, AIA_CUDAF) the way
// the reference's own tests and GUI do, on inputs written by
// tests/test_cpp_classes.py, and writes the results back as raw files.
//
//   glsu_cpp_test <dir>
// <dir>/params.txt : W H nframes radius rate sigma wl wh wi thr
// <dir>/phi0.f64, frames.f32, field.c64 (H*W complex64), aia1..3.bmp
#include <cuda_runtime.h>

#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "glsu_classes.hpp"

template <typename T> static std::vector<T> load(const std::string &p, size_t n)
{
    std::vector<T> v(n);
    std::ifstream in(p, std::ios::binary);
    in.read(reinterpret_cast<char *>(v.data()), sizeof(T) * n);
    if (!in) throw std::runtime_error("cannot read " + p);
    return v;
}

template <typename T> static void save(const std::string &p, const std::vector<T> &v)
{
    std::ofstream out(p, std::ios::binary);
    out.write(reinterpret_cast<const char *>(v.data()), sizeof(T) * v.size());
}

int main(int argc, char **argv)
{
    if (argc < 2) {
        std::cerr << "usage: glsu_cpp_test <dir>\n";
        return 2;
    }
    const std::string dir = argv[1];
    std::ifstream pf(dir + "/params.txt");
    int W, H, nf, r, rr;
    double sigma, wl, wh, wi, thr;
    pf >> W >> H >> nf >> r >> rr >> sigma >> wl >> wh >> wi >> thr;
    const size_t N = (size_t)W * H;
    glsu_wff_params wp{sigma, wl, wh, wi, sigma, wl, wh, wi, thr};
    try {
        // ---- DPRA_CUDAF over a frame sequence (operator(), DPRA_CPU semantics)
        auto phi0d = load<double>(dir + "/phi0.f64", N);
        std::vector<float> phi0f(phi0d.begin(), phi0d.end());
        auto frames = load<float>(dir + "/frames.f32", N * nf);
        std::vector<cv::Mat> mats;
        for (int k = 0; k < nf; k++) {
            cv::Mat m(H, W, cv::CV_32FC1);
            std::copy(frames.begin() + N * k, frames.begin() + N * (k + 1), reinterpret_cast<float *>(m.data));
            mats.push_back(m);
        }
        {
            DPRA::DPRA_CUDAF dpra(phi0f.data(), W, H, rr, r, wp);
            std::vector<std::vector<float>> dphi;
            double t = 0;
            dpra(mats, dphi, t);
            std::vector<float> all;
            for (auto &d : dphi) all.insert(all.end(), d.begin(), d.end());
            save(dir + "/dpra_f32_dphi.f32", all);
            std::vector<float> pc;
            dpra.get_phi_curr(pc);
            save(dir + "/dpra_f32_phicurr.f32", pc);
            std::cout << "DPRA_CUDAF frames=" << dphi.size() << " time_ms=" << t << "\n";
        }
        {
            DPRA::DPRA_CUDA dpra(phi0d.data(), W, H, rr, r, wp);
            std::vector<std::vector<double>> dphi;
            double t = 0;
            dpra(mats, dphi, t);
            std::vector<double> all;
            for (auto &d : dphi) all.insert(all.end(), d.begin(), d.end());
            save(dir + "/dpra_f64_dphi.f64", all);
            std::cout << "DPRA_CUDA frames=" << dphi.size() << " time_ms=" << t << "\n";
        }
        // ---- DPRA_HYBRIDF / DPRA_HYBRID (reference signatures, iNumThreads) against
        //      DPRA_CUDAF / DPRA_CUDA with the same hard-wired window and WFF parameters
        {
            std::vector<std::vector<float>> a, b;
            double t = 0;
            {
                DPRA::DPRA_HYBRIDF hy(phi0f.data(), W, H, rr, 4);
                hy(mats, a, t);
            }
            {
                DPRA::DPRA_CUDAF cu(phi0f.data(), W, H, rr);
                cu(mats, b, t);
            }
            std::vector<std::vector<double>> c, e;
            {
                DPRA::DPRA_HYBRID hy(phi0d.data(), W, H, rr, 4);
                hy(mats, c, t);
            }
            {
                DPRA::DPRA_CUDA cu(phi0d.data(), W, H, rr);
                cu(mats, e, t);
            }
            std::cout << "DPRA_HYBRID equal=" << (a == b && c == e && a.size() == (size_t)nf) << "\n";
        }
        // ---- WFT2_CUDAF (WFF) on a device buffer, as DPRA_CUDAF uses it
        {
            auto f = load<float>(dir + "/field.c64", 2 * N);
            WFT_FPA::WFT::WFT2_DeviceResultsF z;
            WFT_FPA::WFT::WFF2_CUDAF wff(W, H, WFT_FPA::WFT::WFT_TYPE::WFF, (float)sigma, (float)wl, (float)wh,
                                         (float)wi, (float)sigma, (float)wl, (float)wh, (float)wi, (float)thr, z);
            cuFloatComplex *d_f = nullptr;
            cudaMalloc((void **)&d_f, sizeof(cuFloatComplex) * N);
            cudaMemcpy(d_f, f.data(), sizeof(cuFloatComplex) * N, cudaMemcpyHostToDevice);
            double t = 0;
            wff(d_f, z, t);
            std::vector<float> out(2 * N);
            cudaMemcpy(out.data(), z.m_d_filtered, sizeof(cuFloatComplex) * N, cudaMemcpyDeviceToHost);
            cudaFree(d_f);
            save(dir + "/wff_f32.c64", out);
            std::cout << "WFT2_CUDAF time_ms=" << t << "\n";
        }
        // ---- WFT2_CUDAF (WFR) on the same device field: the ridge maps
        {
            auto f = load<float>(dir + "/field.c64", 2 * N);
            WFT_FPA::WFT::WFT2_DeviceResultsF z;
            WFT_FPA::WFT::WFT2_CUDAF wfr(W, H, WFT_FPA::WFT::WFT_TYPE::WFR, (float)sigma, (float)wl, (float)wh,
                                         (float)wi, (float)sigma, (float)wl, (float)wh, (float)wi, 0.f, z);
            cuFloatComplex *d_f = nullptr;
            cudaMalloc((void **)&d_f, sizeof(cuFloatComplex) * N);
            cudaMemcpy(d_f, f.data(), sizeof(cuFloatComplex) * N, cudaMemcpyHostToDevice);
            double t = 0;
            wfr(d_f, z, t);
            const float *maps[8] = {z.m_d_wx, z.m_d_wy, z.m_d_phase, z.m_d_phase_comp,
                                    z.m_d_b,  z.m_d_r,  z.m_d_cxx,   z.m_d_cyy};
            std::vector<float> out(8 * N);
            for (int k = 0; k < 8; k++)
                cudaMemcpy(out.data() + k * N, maps[k], sizeof(float) * N, cudaMemcpyDeviceToHost);
            cudaFree(d_f);
            save(dir + "/wfr_f32.f32", out);
            std::cout << "WFT2_CUDAF(WFR) time_ms=" << t << "\n";
        }
        // ---- AIA_CUDAF on BMP files read through cv::imread
        {
            std::vector<cv::Mat> v;
            for (int k = 1; k <= 3; k++) v.push_back(cv::imread(dir + "/aia" + std::to_string(k) + ".bmp"));
            AIA::AIA_CUDAF aia(v);
            std::vector<float> phi, delta{0.8622f, 0.3188f, -1.3077f};
            double t = 0;
            int it = 0;
            float err = 0;
            aia(phi, delta, t, it, err, v, 20, 1e-4f, 6);
            save(dir + "/aia_phi.f32", phi);
            save(dir + "/aia_delta.f32", delta);
            std::vector<unsigned char> img(v[0].data, v[0].data + (size_t)v[0].rows * v[0].cols);
            save(dir + "/aia_img1.u8", img);
            std::cout << "AIA_CUDAF iters=" << it << " err=" << err << " delta=" << delta[0] << "," << delta[1]
                      << "," << delta[2] << "\n";
        }
        // ---- error behaviour: exceptions instead of exit()/throw int
        int caught = 0;
        try {
            WFT_FPA::WFT::WFT2_DeviceResultsF z;
            WFT_FPA::WFT::WFT2_CUDAF bad(4090, 16, WFT_FPA::WFT::WFT_TYPE::WFR, z);
        } catch (const std::runtime_error &) {
            caught++;
        }
        try {
            WFT_FPA::WFT::WFT2_DeviceResultsF z;
            WFT_FPA::WFT::WFT2_CUDAF bad(4090, 16, WFT_FPA::WFT::WFT_TYPE::WFF, z);
        } catch (const std::runtime_error &e) {
            caught += std::string(e.what()).find("4096") != std::string::npos;
        }
        std::cout << "errors_caught=" << caught << "\n";
    } catch (const std::exception &e) {
        std::cerr << "FAILED: " << e.what() << "\n";
        return 1;
    }
    return 0;
}
