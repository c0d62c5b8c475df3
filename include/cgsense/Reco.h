// cgsense/Reco.h -- C++ drop-in for the reference's reconstruction object.
//
// Same class names, member functions, public buffers and error behaviour as
// expRad/4d_lung's CGSense/Reco.h, Fourier.h and Trajectory.h, for the
// CG-SENSE path: a program written against the reference (CGSense.cpp:27-291)
// compiles against this header instead and runs the operator and solver on
// the GPU through the C ABI of cgsense_c.h.
//
// Differences, all internal to the path:
//   * ConvKernel::weights / indices stay empty: the KB taps are evaluated on
//     the GPU from the trajectory (calculateWeights uploads it).
//   * nufftFWD does not leave the FFT'd grids in `img` (the reference reuses
//     img[c] as scratch, Reco.cpp:529-537).
//   * Buffers from allocData / allocImg / allocSMaps are page-locked host
//     memory (faster transfers); free them only through this class.
//   * Errors print the reference's style of message and call
//     exit(EXIT_FAILURE), as the reference does.
#pragma once
#include <iostream>
#include <string>
#include <vector>

#include "cgsense_c.h"

#ifndef FFTW3_H
typedef float fftwf_complex[2];
#endif

template <class T>
using mat2d = std::vector<std::vector<T>>;

class Reco;

// Trajectory.h:17-41: custom trajectories derive from Trajectory and
// provide calculateTraj(); Reco::setTrajectory is overloaded per type.
class Trajectory {
public:
    Trajectory(Reco* reco) : r(reco) {}
    virtual ~Trajectory() {}
    void calculateKMax();
    void setImportPath(const std::string& s) { importPath = s; }
    mat2d<double> getKMax() { return kmax; }
    virtual void calculateTraj() = 0;
    mat2d<double> kSpaceTraj;

protected:
    Reco* r;
    std::vector<std::vector<double>> kmax;

private:
    std::string importPath;
};

// Trajectory.h:43-80
class WaveCaipi : public Trajectory {
public:
    WaveCaipi(Reco* reco) : Trajectory(reco) {}
    void setNOsc(const int& n) { nOsc = n; }
    void setGradAmp(const double& a) { gradAmp = a; }
    void setAmpCorrY(const double& y) { ampCorrY = y; }
    void setAmpCorrZ(const double& z) { ampCorrZ = z; }
    void setShiftY(const double& y) { shiftY = y; }
    void setShiftZ(const double& z) { shiftZ = z; }
    void setBandwidth(const double& b) { bandwidth = b; }
    void setDwellTime(const double& d) { dwellTime = d; }
    void setPseudoGradAmp(const double& a) { pseudoGradAmp = a; }

    int getNOsc() const { return nOsc; }
    double getGradAmp() const { return gradAmp; }
    double getAmpCorrY() const { return ampCorrY; }
    double getAmpCorrZ() const { return ampCorrZ; }
    double getShiftY() const { return shiftY; }
    double getShiftZ() const { return shiftZ; }
    double getBandwidth() const { return bandwidth; }
    double getDwellTime() const { return dwellTime; }

    virtual void calculateTraj();

private:
    int nOsc = 4;
    double ampCorrY = 1.0;
    double ampCorrZ = 1.0;
    double gradAmp = 0.0;
    double pseudoGradAmp = 0.0;
    double bandwidth = 0.0;
    double shiftY = 0.0;
    double shiftZ = 0.0;
    double dwellTime = 0.0;
};

// Fourier.h:12-54: centred in-place 3-D FFT (GPU).
class Fourier {
public:
    Fourier(const int& x, const int& y, const int& z) : sizeX(x), sizeY(y), sizeZ(z) {}
    ~Fourier();
    void initFT();
    void transformFWD(fftwf_complex* a) const;
    void transformBWD(fftwf_complex* a, bool rescale = true) const;
    void setSizeX(const int& x) { sizeX = x; }
    void setSizeY(const int& y) { sizeY = y; }
    void setSizeZ(const int& z) { sizeZ = z; }
    void setWisdomFileName(const std::string& s) { wisdomFileName = s; }

private:
    int sizeX, sizeY, sizeZ;
    std::string wisdomFileName;
    mutable cgs_ctx* ctx = nullptr;
    cgs_ctx* context() const;
};

class Reco {
public:
    enum class Density { NONE, VORONOI3D, IMPORT, UNDEFINED };
    Reco();
    ~Reco();

    // Reco.h:26-75
    class ConvKernel {
    public:
        ConvKernel(Reco* r) : reco(r), kernelFT(nullptr) {}
        ~ConvKernel();
        void calculateWeights();
        void calculateKernelFT();
        void clearWeights();
        void excludeMissingData();
        float getB() const { return b; }
        float getW() const { return w; }
        int getKernelOrder() const { return kernelOrder; }
        void setB(const float& b1) { b = b1; }
        void setW(const float& w1) { w = w1; }
        void setKernelOrder(const int& a) { kernelOrder = a; }
        mat2d<float> weights;   // stays empty: taps are evaluated on the GPU
        mat2d<int> indices;     // stays empty
        fftwf_complex* kernelFT;

    private:
        friend class Reco;
        Reco* reco;
        float b = 14.9086f;
        float w = 4.25f;
        int kernelOrder = 5;
    };

    ConvKernel* kernel;
    Trajectory* trajectory;
    Fourier* ft;

    fftwf_complex* data;
    fftwf_complex* dataBuffer;
    std::vector<fftwf_complex*> sMaps;
    std::vector<float> denCorr;
    std::vector<int> numPerformedCGIterations;
    std::vector<double> cgResiduals;
    std::vector<fftwf_complex*> img;
    fftwf_complex* cgSenseImg;

    void check();
    void init();
    void finalize();
    bool importParameters(const std::string& path);
    bool createLogFile(const std::string& path);
    bool setDataInputPaths();

    void cgSenseDynamic();

    static int indexTransform(const int& i, const int& j, const int& k, const int& ni, const int& nj, const int& nk)
    {
        return k + nk * j + nk * nj * i;
    }

    void setTrajectory(WaveCaipi* t);
    void setSampling(const int& x, const int& y, const int& z) { sX = x; sY = y; sZ = z; }
    void setSX(const int& x) { sX = x; }
    void setSY(const int& y) { sY = y; }
    void setSZ(const int& z) { sZ = z; }
    void setNCh(const int& n) { nCh = n; }
    void setGridSize(const int& x, const int& y, const int& z) { gridSizeX = x; gridSizeY = y; gridSizeZ = z; }
    void setGridSizeX(const int& x) { gridSizeX = x; }
    void setGridSizeY(const int& y) { gridSizeY = y; }
    void setGridSizeZ(const int& z) { gridSizeZ = z; }
    void setOffcenter(const int& x, const int& y, const int& z) { offcenterX = x; offcenterY = y; offcenterZ = z; }
    void setOffcenterX(const int& x) { offcenterX = x; }
    void setOffcenterY(const int& y) { offcenterY = y; }
    void setOffcenterZ(const int& z) { offcenterZ = z; }
    void setFovY(const double& d) { fovY = d; }
    void setFovZ(const double& d) { fovZ = d; }
    void setCGThreshold(const double& x) { cgThreshold = x; }
    void setBatch(const int& b) { batch = b; }
    void setBatchFiles(const std::vector<std::string>& s) { batchFiles = s; }
    void setDensityCorrection(const Density& d) { density = d; }
    void setDensityCorrectionPath(const std::string& s) { densityCorrPath = s; }
    void setOutputParentDir(const std::string& s) { outputParentDir = s; }
    void setNumThreads(const int& n) { numThreads = n; }

    int getSX() const { return sX; }
    int getSY() const { return sY; }
    int getSZ() const { return sZ; }
    int getNCh() const { return nCh; }
    int getGridSizeX() const { return gridSizeX; }
    int getGridSizeY() const { return gridSizeY; }
    int getGridSizeZ() const { return gridSizeZ; }
    int getOffcenterX() const { return offcenterX; }
    int getOffcenterY() const { return offcenterY; }
    int getOffcenterZ() const { return offcenterZ; }
    int getBatch() const { return batch; }
    int getBatchSize() const { return (int)batchFiles.size(); }
    std::string getBatchFileNum(const int& n) const { return batchFiles[n]; }
    std::vector<std::string> getBatchFiles() { return batchFiles; }
    double getFovY() const { return fovY; }
    double getFovZ() const { return fovZ; }
    double getCGThreshold() const { return cgThreshold; }
    int getTotalGridSize() const { return totalGridSize; }
    int getNumThreads() const { return numThreads; }
    int getNumThreadsFFTW() const { return numThreadsFFTW; }
    Density getDensityCorrection() const { return density; }
    std::string getDensityCorrectionPath() const { return densityCorrPath; }
    std::string getOutputParentDir() const { return outputParentDir; }

    void allocImg();
    void allocData(fftwf_complex** d);
    void allocSMaps();
    void freeImg();

    void nufftFWD();
    void nufftBWD();

    // Extension: the underlying C ABI context (created by calculateWeights).
    cgs_ctx* context() const { return ctx; }

private:
    friend class Trajectory;
    friend class WaveCaipi;
    cgs_ctx* context_or_die();
    void die(int status, const char* where) const;

    int sX = 0, sY = 0, sZ = 0;
    int nCh = 0;
    int batch = 0;
    double fovY = 0.0, fovZ = 0.0;
    int gridSizeX = 0, gridSizeY = 0, gridSizeZ = 0;
    double cgThreshold = -1;
    int totalGridSize = 0;
    int offcenterX = 0, offcenterY = 0, offcenterZ = 0;
    int numThreads = 32;
    int numThreadsFFTW = 1;
    Density density = Density::NONE;
    std::string outputParentDir;
    std::string densityCorrPath;
    std::vector<std::string> batchFiles;
    // file name parts of setDataInputPaths (Reco.h:207-209, Reco.cpp:15)
    std::string dataPathRoot;
    std::string dataPathFileName;
    std::string dataPathFileExtension = ".bin";
    cgs_ctx* ctx = nullptr;
    fftwf_complex* imgBlock = nullptr;
    fftwf_complex* mapBlock = nullptr;
    std::vector<void*> hostAllocs;
};

// functions.h:319-335
void performDensityCorrection(const Reco& r, fftwf_complex* data, const std::vector<float>& d,
                              const int& nSamplesPerCh, const int& nChannels, const int& nThreads = 1);
