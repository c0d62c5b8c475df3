// reco_shim.cpp -- the C++ drop-in classes of include/cgsense/Reco.h
// (Reco, Reco::ConvKernel, Fourier, Trajectory, WaveCaipi) over the C ABI.
//
// Each member keeps the reference's name, arguments, console messages and
// exit-on-error behaviour (Reco.cpp, Fourier.cpp, Trajectory.cpp); the work
// itself runs on the GPU.
#include "cgsense/Reco.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>

namespace {

const double kGammaBar = 4.257748059639612e7;   // globalVars.h:4

[[noreturn]] void die_msg(const std::string& msg)
{
    std::cout << "\nError: " << msg << "\n";
    std::exit(EXIT_FAILURE);
}

void check_status(cgs_ctx* ctx, int st, const char* where)
{
    if (st == CGS_OK) return;
    std::string m = std::string(where) + ": " + (ctx ? cgs_last_error(ctx) : "invalid call");
    die_msg(m);
}

fftwf_complex* alloc_complex(size_t n)
{
    return reinterpret_cast<fftwf_complex*>(cgs_alloc_host(n * sizeof(fftwf_complex)));
}

}  // namespace

// ---------------------------------------------------------------------------
// Trajectory / WaveCaipi (Trajectory.cpp:9-184)
// ---------------------------------------------------------------------------

void Trajectory::calculateKMax()
{
    kmax = {
        {0.0, 1.0},
        {r->sY / (double)(r->fovY * 2.0 * kGammaBar), -r->sY / (double)(r->fovY * 2.0 * kGammaBar)},
        {r->sZ / (double)(r->fovZ * 2.0 * kGammaBar), -r->sZ / (double)(r->fovZ * 2.0 * kGammaBar)},
    };
}

void WaveCaipi::calculateTraj()
{
    std::cout << "Calculating wave-CAIPI trajectory...\n";
    cgs_wave w;
    w.sx = r->sX;
    w.sy = r->sY;
    w.sz = r->sZ;
    w.gx = r->gridSizeX;
    w.gy = r->gridSizeY;
    w.gz = r->gridSizeZ;
    w.fov_y = r->fovY;
    w.fov_z = r->fovZ;
    w.n_osc = nOsc;
    w.grad_amp = gradAmp;
    w.amp_corr_y = ampCorrY;
    w.amp_corr_z = ampCorrZ;
    w.shift_y = shiftY;
    w.shift_z = shiftZ;
    w.dwell = dwellTime;
    const size_t n = (size_t)r->sX * r->sY * r->sZ;
    std::vector<double> k(3 * n);
    if (cgs_wave_caipi(&w, k.data()) != CGS_OK) die_msg("invalid wave-CAIPI parameters");
    kSpaceTraj.assign(n, std::vector<double>(3));
    for (size_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) kSpaceTraj[i][a] = k[3 * i + a];
    std::cout << "Finished calculating trajectory\n";
}

// ---------------------------------------------------------------------------
// Fourier (Fourier.cpp:4-42)
// ---------------------------------------------------------------------------

Fourier::~Fourier()
{
    if (ctx) cgs_destroy(ctx);
}

cgs_ctx* Fourier::context() const
{
    if (!ctx) {
        cgs_params p;
        cgs_default_params(&p);
        p.img[0] = p.grid[0] = sizeX;
        p.img[1] = p.grid[1] = sizeY;
        p.img[2] = p.grid[2] = sizeZ;
        p.n_ch = 1;
        check_status(nullptr, cgs_create(&p, &ctx), "Fourier::initFT");
    }
    return ctx;
}

void Fourier::initFT() { context(); }

void Fourier::transformFWD(fftwf_complex* a) const
{
    check_status(context(), cgs_fft3(context(), &a[0][0], -1, 0), "Fourier::transformFWD");
}

void Fourier::transformBWD(fftwf_complex* a, bool rescale) const
{
    check_status(context(), cgs_fft3(context(), &a[0][0], +1, rescale ? 1 : 0), "Fourier::transformBWD");
}

// ---------------------------------------------------------------------------
// Reco
// ---------------------------------------------------------------------------

Reco::Reco()
    : kernel(nullptr), trajectory(nullptr), ft(nullptr), data(nullptr), dataBuffer(nullptr), cgSenseImg(nullptr)
{
}

Reco::~Reco()
{
    delete kernel;
    delete ft;
    for (void* p : hostAllocs) cgs_free_host(p);
    if (ctx) cgs_destroy(ctx);
}

void Reco::die(int status, const char* where) const { check_status(ctx, status, where); }

cgs_ctx* Reco::context_or_die()
{
    if (ctx) return ctx;
    if (!kernel) die_msg("Reco::init has not been called");
    cgs_params p;
    cgs_default_params(&p);
    p.img[0] = p.grid[0] = gridSizeX;
    p.img[1] = p.grid[1] = gridSizeY;
    p.img[2] = p.grid[2] = gridSizeZ;
    p.n_ch = nCh;
    p.kb_b = kernel->b;
    p.kb_w = kernel->w;
    p.kb_order = kernel->kernelOrder;
    const int st = cgs_create(&p, &ctx);
    if (st != CGS_OK) die_msg("could not create the GPU reconstruction context (status " + std::to_string(st) + ")");
    return ctx;
}

void Reco::setTrajectory(WaveCaipi* t)
{
    t->calculateKMax();
    t->calculateTraj();
    trajectory = t;
    if (trajectory == nullptr) die_msg("Trajectory conversion failed in setTrajectory!");
}

bool Reco::createLogFile(const std::string&) { return true; }
bool Reco::importParameters(const std::string&) { return true; }
// Reco.cpp:63-71: one state file per batch entry,
// root + file name + index + extension
bool Reco::setDataInputPaths()
{
    for (int i = 0; i < batch; i++)
        batchFiles.push_back(dataPathRoot + dataPathFileName + std::to_string(i) + dataPathFileExtension);
    return true;
}

void Reco::check()
{
    if (!batchFiles.empty()) {
        std::cout << "Checking all files...";
        for (const auto& path : batchFiles) {
            std::FILE* f = std::fopen(path.c_str(), "rb");
            if (!f) die_msg("Could not open binary data file " + path);
            std::fclose(f);
        }
        std::cout << " Done!\n";
    }
}

void Reco::init()
{
    kernel = new ConvKernel(this);
    kernel->setB(14.9086f);
    kernel->setW(4.25f);
    kernel->setKernelOrder(5);
    ft = new Fourier(gridSizeX, gridSizeY, gridSizeZ);
    sMaps.assign(nCh, nullptr);
    totalGridSize = gridSizeX * gridSizeY * gridSizeZ;
    batch = (int)batchFiles.size();
}

void Reco::finalize()
{
    std::string dir = outputParentDir;
    if (!dir.empty() && dir.back() != '/' && dir.back() != '\\') dir += "/";
    std::ofstream os((dir + "results/performedIterations.txt").c_str());
    for (int n : numPerformedCGIterations) os << n << "\n";
}

void Reco::allocData(fftwf_complex** d)
{
    *d = alloc_complex((size_t)sX * sY * sZ * nCh);
    hostAllocs.push_back(*d);
}

void Reco::allocImg()
{
    if (!imgBlock) {
        imgBlock = alloc_complex((size_t)nCh * totalGridSize);
        hostAllocs.push_back(imgBlock);
    }
    img.resize(nCh);
    for (int c = 0; c < nCh; ++c) img[c] = imgBlock + (size_t)c * totalGridSize;
}

void Reco::allocSMaps()
{
    if (!mapBlock) {
        mapBlock = alloc_complex((size_t)nCh * totalGridSize);
        hostAllocs.push_back(mapBlock);
    }
    sMaps.resize(nCh);
    for (int c = 0; c < nCh; ++c) sMaps[c] = mapBlock + (size_t)c * totalGridSize;
}

void Reco::freeImg()
{
    img.clear();
    img.shrink_to_fit();
}

// per-coil pointer arrays -> one contiguous [nCh][N] block (copied only when
// the caller did not use allocImg / allocSMaps)
static const float* contiguous(const std::vector<fftwf_complex*>& v, fftwf_complex* block, size_t n,
                               std::vector<float>& staging)
{
    bool ok = block != nullptr;
    for (size_t c = 0; ok && c < v.size(); ++c) ok = v[c] == block + c * n;
    if (ok) return &block[0][0];
    staging.resize(2 * n * v.size());
    for (size_t c = 0; c < v.size(); ++c) std::memcpy(&staging[2 * n * c], v[c], n * sizeof(fftwf_complex));
    return staging.data();
}

void Reco::nufftBWD()
{
    if (data == nullptr) die_msg("in nufftBWD function: data is NULL pointer!");
    cgs_ctx* c = context_or_die();
    if ((int)img.size() != nCh) allocImg();
    std::vector<float> staging;
    const float* dst = contiguous(img, imgBlock, totalGridSize, staging);
    die(cgs_nufft_adj(c, &data[0][0], const_cast<float*>(dst)), "nufftBWD");
    if (dst == staging.data())
        for (int ch = 0; ch < nCh; ++ch)
            std::memcpy(img[ch], &staging[2 * (size_t)totalGridSize * ch], totalGridSize * sizeof(fftwf_complex));
}

void Reco::nufftFWD()
{
    cgs_ctx* c = context_or_die();
    std::vector<float> staging;
    const float* src = contiguous(img, imgBlock, totalGridSize, staging);
    die(cgs_nufft_fwd(c, src, &data[0][0]), "nufftFWD");
}

void Reco::cgSenseDynamic()
{
    if (cgSenseImg) cgs_free_host(cgSenseImg);
    cgSenseImg = alloc_complex(totalGridSize);
    if (cgThreshold == -1) die_msg("no threshold set for CG SENSE!");
    cgs_ctx* c = context_or_die();
    std::vector<float> s1, s2;
    die(cgs_set_smaps(c, contiguous(sMaps, mapBlock, totalGridSize, s1)), "cgSense");
    die(cgs_set_dcf(c, denCorr.empty() ? nullptr : denCorr.data()), "cgSense");
    cgResiduals.clear();
    std::cout << "Begin cgSense\n";
    const int maxIter = 16;   // Reco.cpp:228,308-309
    std::vector<double> res(maxIter);
    int32_t iters = 0;
    const int st = cgs_cg_solve_images(c, contiguous(img, imgBlock, totalGridSize, s2), &cgSenseImg[0][0],
                                       cgThreshold, maxIter, res.data(), &iters);
    if (st == CGS_ERR_NONFINITE) {
        std::cout << "\nError in function cgSense: NaN or INF value in image detected!\n";
        std::exit(EXIT_FAILURE);
    }
    die(st, "cgSense");
    for (int i = 0; i < iters; ++i) {
        cgResiduals.push_back(res[i]);
        std::cout << "\n\tIteration:\t" << i << "\t" << res[i] << "\t" << cgThreshold << "\n";
    }
    numPerformedCGIterations.push_back(iters);
    std::cout << "\nEnd cgSense\n";
}

// ---------------------------------------------------------------------------
// Reco::ConvKernel
// ---------------------------------------------------------------------------

Reco::ConvKernel::~ConvKernel()
{
    if (kernelFT) cgs_free_host(kernelFT);
}

void Reco::ConvKernel::calculateWeights()
{
    std::cout << "Calculating kernel weights for each grid point\n";
    cgs_ctx* c = reco->context_or_die();
    if (!reco->trajectory) die_msg("no trajectory set");
    const auto& kt = reco->trajectory->kSpaceTraj;
    std::vector<double> k(3 * kt.size());
    for (size_t i = 0; i < kt.size(); ++i)
        for (int a = 0; a < 3; ++a) k[3 * i + a] = kt[i][a];
    check_status(c, cgs_set_trajectory(c, k.data(), (int64_t)kt.size()), "calculateWeights");
    std::cout << "Finished calculating kernel weights\n";
}

void Reco::ConvKernel::calculateKernelFT()
{
    cgs_ctx* c = reco->context_or_die();
    if (!kernelFT)
        kernelFT = alloc_complex((size_t)reco->gridSizeX * reco->gridSizeY * reco->gridSizeZ);
    check_status(c, cgs_kernel_ft(c, &kernelFT[0][0]), "calculateKernelFT");
}

void Reco::ConvKernel::clearWeights()
{
    weights.clear();
    indices.clear();
}

void Reco::ConvKernel::excludeMissingData()
{
    cgs_ctx* c = reco->context_or_die();
    check_status(c, cgs_mask_from_data(c, &reco->data[0][0]), "excludeMissingData");
}

// functions.h:319-335
void performDensityCorrection(const Reco&, fftwf_complex* data, const std::vector<float>& d,
                              const int& nSamplesPerCh, const int& nChannels, const int&)
{
    if (d.empty()) return;
    const int dSize = (int)d.size();
    (void)nSamplesPerCh;
    for (int ch = 0; ch < nChannels; ++ch)
        for (int i = 0; i < dSize; ++i) {
            data[(size_t)ch * dSize + i][0] *= d[i];
            data[(size_t)ch * dSize + i][1] *= d[i];
        }
}
