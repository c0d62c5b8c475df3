// ref_driver.cpp -- a command-line driver around the reference's own CG-SENSE
// hot path, compiled from the unmodified reference sources (Reco.cpp,
// Fourier.cpp, Trajectory.cpp, IO.cpp of expRad/4d_lung CGSense).
//
// TEST INFRASTRUCTURE: used only to pin the oracle and to generate golden
// fixtures.  The reference's own main (CGSense.cpp:27-291) needs windows.h and
// CGAL, so this file replaces it.  Every mode mirrors a step of that main:
//
//   traj      WaveCaipi::calculateTraj              (CGSense.cpp:51-61)
//   taps      ConvKernel::calculateWeights + excludeMissingData
//                                                   (CGSense.cpp:163,224)
//   kernelft  ConvKernel::calculateKernelFT          (CGSense.cpp:147-154)
//   fwd       Reco::nufftFWD on given coil grids     (Reco.cpp:521-553)
//   bwd       Reco::nufftBWD on given samples        (Reco.cpp:468-519)
//   cg        weights, exclude, density, nufftBWD, cgSenseDynamic
//                                                   (CGSense.cpp:218-266)
//   io        IO::importDataBin / importSensitivityMaps / exportFFTWComplexBin
//
// Usage: ref_driver <mode> <dir>.  <dir>/params.txt holds "key value" lines;
// arrays are raw little-endian binaries in <dir>; outputs are written there.
// The reference keeps grid-size-dependent `static` locals in convFunction
// (Reco.h:221-226), so one process handles one grid size.
#include "Reco.h"
#include "IO.h"
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>
#include <omp.h>

namespace {

std::map<std::string, std::string> g_params;

void load_params(const std::string& dir)
{
    std::ifstream f(dir + "/params.txt");
    if (!f) { std::fprintf(stderr, "ref_driver: no params.txt in %s\n", dir.c_str()); std::exit(2); }
    std::string k, v;
    while (f >> k >> v) g_params[k] = v;
}

double pd(const char* k, double def)
{
    auto it = g_params.find(k);
    return it == g_params.end() ? def : std::stod(it->second);
}
int pi(const char* k, int def)
{
    auto it = g_params.find(k);
    return it == g_params.end() ? def : std::stoi(it->second);
}

template <class T>
std::vector<T> read_bin(const std::string& path, size_t n, bool required = true)
{
    std::vector<T> v;
    std::FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
        if (required) { std::fprintf(stderr, "ref_driver: cannot open %s\n", path.c_str()); std::exit(2); }
        return v;
    }
    v.resize(n);
    size_t got = std::fread(v.data(), sizeof(T), n, f);
    std::fclose(f);
    if (got != n) { std::fprintf(stderr, "ref_driver: short read %s (%zu of %zu)\n", path.c_str(), got, n); std::exit(2); }
    return v;
}

template <class T>
void write_bin(const std::string& path, const T* p, size_t n)
{
    std::FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) { std::fprintf(stderr, "ref_driver: cannot write %s\n", path.c_str()); std::exit(2); }
    std::fwrite(p, sizeof(T), n, f);
    std::fclose(f);
}

// A Trajectory plug-in (Trajectory.h:1-4: custom trajectories derive from the
// Trajectory class) that hands a precomputed k-space trajectory to Reco.
class InjectedTrajectory : public WaveCaipi {
public:
    InjectedTrajectory(Reco* r, const std::vector<double>& k) : WaveCaipi(r), k_(k) {}
    void calculateTraj() override
    {
        const size_t n = k_.size() / 3;
        kSpaceTraj.assign(n, std::vector<double>(3));
        for (size_t i = 0; i < n; ++i)
            for (int a = 0; a < 3; ++a) kSpaceTraj[i][a] = k_[3 * i + a];
    }
private:
    std::vector<double> k_;
};

void setup_reco(Reco& reco)
{
    reco.setGridSize(pi("gx", 0), pi("gy", 0), pi("gz", 0));
    reco.setSampling(pi("sx", 1), pi("sy", 1), pi("sz", 1));
    reco.setNCh(pi("nch", 1));
    reco.setFovY(pd("fovy", 1.0));
    reco.setFovZ(pd("fovz", 1.0));
    reco.setCGThreshold(pd("cg_threshold", 0.0));
    reco.setDensityCorrection(Reco::Density::NONE);
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc < 3) { std::fprintf(stderr, "usage: ref_driver <mode> <dir>\n"); return 2; }
    const std::string mode = argv[1];
    const std::string dir = argv[2];
    load_params(dir);
    const int nthreads = pi("threads", omp_get_max_threads());
    omp_set_num_threads(nthreads);

    Reco reco;
    setup_reco(reco);
    reco.setNumThreads(nthreads);

    const int nS = reco.getSX() * reco.getSY() * reco.getSZ();
    const int nCh = reco.getNCh();
    const int Ng = reco.getGridSizeX() * reco.getGridSizeY() * reco.getGridSizeZ();

    if (mode == "traj") {
        WaveCaipi* wc = new WaveCaipi(&reco);
        wc->setNOsc(pi("nosc", 4));
        wc->setDwellTime(pd("dwell", 6.3e-6));
        wc->setGradAmp(pd("grad_amp", 0.006));
        wc->setBandwidth(pd("bandwidth", 350));
        wc->setAmpCorrY(pd("amp_corr_y", 0.998));
        wc->setAmpCorrZ(pd("amp_corr_z", 1.01));
        wc->setShiftY(pd("shift_y", 5.6e-6));
        wc->setShiftZ(pd("shift_z", 6.5e-6));
        reco.setTrajectory(wc);
        std::vector<double> out((size_t)nS * 3);
        for (int i = 0; i < nS; ++i)
            for (int a = 0; a < 3; ++a) out[3 * (size_t)i + a] = reco.trajectory->kSpaceTraj[i][a];
        write_bin(dir + "/traj_out.bin", out.data(), out.size());
        return 0;
    }

    if (mode == "io") {
        // IO::importDataBin permutes readout-fastest file order to z-fastest
        // memory order (IO.cpp:55-98); importSensitivityMaps reads map<c>.bin.
        reco.init();
        reco.allocData(&reco.data);
        IO::importDataBin(reco, reco.data, dir + "/raw_file.bin");
        write_bin(dir + "/io_data_out.bin", &reco.data[0][0], (size_t)nS * nCh * 2);
        reco.allocSMaps();
        IO::importSensitivityMaps(reco.sMaps, Ng, nCh, dir + "/");
        std::vector<float> maps((size_t)Ng * nCh * 2);
        for (int c = 0; c < nCh; ++c)
            std::copy(&reco.sMaps[c][0][0], &reco.sMaps[c][0][0] + (size_t)Ng * 2, maps.begin() + (size_t)c * Ng * 2);
        write_bin(dir + "/io_maps_out.bin", maps.data(), maps.size());
        IO::exportFFTWComplexBin(reco.sMaps[0], dir + "/io_export.bin", Ng);
        return 0;
    }

    // All remaining modes use an injected trajectory.
    std::vector<double> k = read_bin<double>(dir + "/traj.bin", (size_t)nS * 3);
    InjectedTrajectory* tr = new InjectedTrajectory(&reco, k);
    reco.setTrajectory(tr);
    reco.init();
    reco.ft->initFT();

    if (mode == "kernelft") {
        reco.kernel->calculateKernelFT();
        write_bin(dir + "/kernelft_out.bin", &reco.kernel->kernelFT[0][0], (size_t)Ng * 2);
        return 0;
    }

    reco.allocData(&reco.data);
    std::vector<float> data = read_bin<float>(dir + "/data.bin", (size_t)nS * nCh * 2, mode != "fwd" && mode != "taps");
    if (!data.empty()) std::copy(data.begin(), data.end(), &reco.data[0][0]);

    reco.kernel->calculateWeights();
    if (!data.empty()) reco.kernel->excludeMissingData();

    if (mode == "taps") {
        std::vector<int> cnt(nS), idx;
        std::vector<float> w;
        for (int i = 0; i < nS; ++i) {
            cnt[i] = (int)reco.kernel->indices[i].size();
            idx.insert(idx.end(), reco.kernel->indices[i].begin(), reco.kernel->indices[i].end());
            w.insert(w.end(), reco.kernel->weights[i].begin(), reco.kernel->weights[i].end());
        }
        write_bin(dir + "/tap_count_out.bin", cnt.data(), cnt.size());
        write_bin(dir + "/tap_idx_out.bin", idx.data(), idx.size());
        write_bin(dir + "/tap_w_out.bin", w.data(), w.size());
        return 0;
    }

    reco.kernel->calculateKernelFT();
    reco.allocImg();

    if (mode == "fwd") {
        std::vector<float> img = read_bin<float>(dir + "/img.bin", (size_t)Ng * nCh * 2);
        for (int c = 0; c < nCh; ++c)
            std::copy(img.begin() + (size_t)c * Ng * 2, img.begin() + (size_t)(c + 1) * Ng * 2, &reco.img[c][0][0]);
        reco.nufftFWD();
        write_bin(dir + "/data_out.bin", &reco.data[0][0], (size_t)nS * nCh * 2);
        return 0;
    }

    // Density weights D (IMPORT mode, IO.cpp:129-156), applied to the measured
    // samples as performDensityCorrection does (functions.h:319-335).  That
    // function sits in functions.h, which needs CGAL, so the six-line loop is
    // repeated here and the vector is handed to Reco exactly as CGSense.cpp:178.
    std::vector<float> dcf = read_bin<float>(dir + "/dcf.bin", (size_t)nS, false);
    if (!dcf.empty()) {
        reco.denCorr = dcf;
        for (int c = 0; c < nCh; ++c)
            for (int i = 0; i < nS; ++i) {
                reco.data[(size_t)c * nS + i][0] *= dcf[i];
                reco.data[(size_t)c * nS + i][1] *= dcf[i];
            }
    }

    if (mode == "bwd") {
        reco.nufftBWD();
        std::vector<float> img((size_t)Ng * nCh * 2);
        for (int c = 0; c < nCh; ++c)
            std::copy(&reco.img[c][0][0], &reco.img[c][0][0] + (size_t)Ng * 2, img.begin() + (size_t)c * Ng * 2);
        write_bin(dir + "/img_out.bin", img.data(), img.size());
        return 0;
    }

    if (mode == "cg") {
        reco.nufftBWD();
        reco.allocSMaps();
        std::vector<float> maps = read_bin<float>(dir + "/smaps.bin", (size_t)Ng * nCh * 2);
        for (int c = 0; c < nCh; ++c)
            std::copy(maps.begin() + (size_t)c * Ng * 2, maps.begin() + (size_t)(c + 1) * Ng * 2, &reco.sMaps[c][0][0]);
        double t0 = omp_get_wtime();
        reco.cgSenseDynamic();
        double t1 = omp_get_wtime();
        write_bin(dir + "/x_out.bin", &reco.cgSenseImg[0][0], (size_t)Ng * 2);
        write_bin(dir + "/residuals_out.bin", reco.cgResiduals.data(), reco.cgResiduals.size());
        int iters = reco.numPerformedCGIterations.empty() ? 0 : reco.numPerformedCGIterations.back();
        write_bin(dir + "/iters_out.bin", &iters, 1);
        double secs = t1 - t0;
        write_bin(dir + "/cg_seconds_out.bin", &secs, 1);
        return 0;
    }

    std::fprintf(stderr, "ref_driver: unknown mode %s\n", mode.c_str());
    return 2;
}
