// reco_dropin.cpp -- a reconstruction program written against the
// reference's Reco interface (the flow of CGSense.cpp:42-266 for one state
// file), compiled against include/cgsense/Reco.h and linked with
// libcgsense.so.  Used by tests/test_dropin.py.
//
// Usage: reco_dropin <dir>; <dir>/params.txt holds "gx gy gz ns nch
// threshold"; inputs traj.bin (double [ns][3]), data.bin (complex64
// [nch][ns]), dcf.bin (float [ns]), smaps.bin (complex64 [nch][grid]);
// outputs x_out.bin, residuals_out.bin, iters_out.bin, bwd_out.bin.
#include "cgsense/Reco.h"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

// A custom trajectory plug-in (Trajectory.h:1-4): the k-space coordinates
// come from a file instead of the wave-CAIPI model.
class FileTrajectory : public WaveCaipi {
public:
    FileTrajectory(Reco* r, std::vector<double> k) : WaveCaipi(r), k_(std::move(k)) {}
    void calculateTraj() override
    {
        kSpaceTraj.assign(k_.size() / 3, std::vector<double>(3));
        for (size_t i = 0; i < k_.size() / 3; ++i)
            for (int a = 0; a < 3; ++a) kSpaceTraj[i][a] = k_[3 * i + a];
    }

private:
    std::vector<double> k_;
};

template <class T>
static std::vector<T> load(const std::string& p, size_t n)
{
    std::vector<T> v(n);
    std::FILE* f = std::fopen(p.c_str(), "rb");
    if (!f || std::fread(v.data(), sizeof(T), n, f) != n) {
        std::fprintf(stderr, "cannot read %s\n", p.c_str());
        std::exit(2);
    }
    std::fclose(f);
    return v;
}

template <class T>
static void save(const std::string& p, const T* d, size_t n)
{
    std::FILE* f = std::fopen(p.c_str(), "wb");
    std::fwrite(d, sizeof(T), n, f);
    std::fclose(f);
}

int main(int argc, char** argv)
{
    if (argc < 2) return 2;
    const std::string dir = argv[1];
    int gx, gy, gz, ns, nch;
    double thr;
    std::ifstream pf(dir + "/params.txt");
    pf >> gx >> gy >> gz >> ns >> nch >> thr;

    Reco reco;
    reco.setGridSize(gx, gy, gz);
    reco.setSampling(ns, 1, 1);
    reco.setNCh(nch);
    reco.setFovY(1.0);
    reco.setFovZ(1.0);
    FileTrajectory* tr = new FileTrajectory(&reco, load<double>(dir + "/traj.bin", 3 * (size_t)ns));
    reco.setTrajectory(tr);
    reco.setDensityCorrection(Reco::Density::IMPORT);
    reco.setCGThreshold(thr);
    reco.init();
    reco.check();
    reco.allocData(&reco.data);
    std::vector<float> data = load<float>(dir + "/data.bin", 2 * (size_t)ns * nch);
    std::copy(data.begin(), data.end(), &reco.data[0][0]);
    reco.kernel->calculateWeights();
    reco.kernel->calculateKernelFT();
    reco.kernel->excludeMissingData();
    reco.denCorr = load<float>(dir + "/dcf.bin", ns);
    performDensityCorrection(reco, reco.data, reco.denCorr, ns, nch, 1);
    reco.allocImg();
    reco.nufftBWD();
    const size_t ng = (size_t)gx * gy * gz;
    save(dir + "/bwd_out.bin", &reco.img[0][0][0], 2 * ng * nch);
    reco.allocSMaps();
    std::vector<float> maps = load<float>(dir + "/smaps.bin", 2 * ng * nch);
    for (int c = 0; c < nch; ++c) std::copy(maps.begin() + 2 * ng * c, maps.begin() + 2 * ng * (c + 1), &reco.sMaps[c][0][0]);
    reco.cgSenseDynamic();
    save(dir + "/x_out.bin", &reco.cgSenseImg[0][0], 2 * ng);
    save(dir + "/residuals_out.bin", reco.cgResiduals.data(), reco.cgResiduals.size());
    int it = reco.numPerformedCGIterations.back();
    save(dir + "/iters_out.bin", &it, 1);
    save(dir + "/kernelft_out.bin", &reco.kernel->kernelFT[0][0], 2 * ng);
    delete tr;
    return 0;
}
