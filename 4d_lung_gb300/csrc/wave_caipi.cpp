// wave_caipi.cpp -- the wave-CAIPI ("corkscrew") trajectory of the
// reference's Trajectory plug-in (WaveCaipi::calculateTraj with
// Trajectory::calculateKMax, Trajectory.cpp:9-184; constants globalVars.h:3-4).
//
// One-off host computation (double precision): the sinusoidal Gy/Gz
// gradients are integrated on a 10 us raster oversampled 10^4 times with the
// trapezoid rule, sampled at the ADC times with the per-axis delays, placed
// on the ky/kz base lines, normalised to [0,1] with a 42-cell border and
// permuted to the z-fastest sample order.  The steps and constants are those
// of the reference, so that the same parameters give the same k-space
// coordinates.
#include "cgsense_c.h"

#include <algorithm>
#include <cmath>
#include <vector>

extern "C" int cgs_wave_caipi(const cgs_wave* w, double* k_out)
{
    if (!w || !k_out) return CGS_ERR_ARG;
    if (w->sx < 2 || w->sy < 2 || w->sz < 2 || w->n_osc < 1 || w->gx < 1 || w->gy < 1 || w->gz < 1 ||
        !(w->dwell > 0) || !(w->fov_y > 0) || !(w->fov_z > 0))
        return CGS_ERR_ARG;
    const double PI_REF = 3.14159265359;                      // globalVars.h:3
    const double gammaBar = 4.257748059639612 * std::pow(10, 7);  // globalVars.h:4
    const int sX = w->sx, sY = w->sy, sZ = w->sz, nOsc = w->n_osc;
    const double kmax[3][2] = {
        {0.0, 1.0},
        {sY / (double)(w->fov_y * 2.0 * gammaBar), -sY / (double)(w->fov_y * 2.0 * gammaBar)},
        {sZ / (double)(w->fov_z * 2.0 * gammaBar), -sZ / (double)(w->fov_z * 2.0 * gammaBar)},
    };
    const double tADC = w->dwell * sX;
    const double gradRasterTime = 10 * std::pow(10, -6);
    const int os = 10000;
    const double dtOs = gradRasterTime / (double)os;
    const int gradSamples = (int)(tADC / gradRasterTime);
    const int gradSamplesZ = (int)((tADC + 0.5 * tADC / (double)nOsc) / gradRasterTime);
    if (gradSamples < 1 || gradSamplesZ < 1) return CGS_ERR_ARG;
    const long long nSamples = (long long)sX * sY * sZ;
    const double sinTerm = std::pow(std::sin(nOsc * PI_REF / (double)(2 * nOsc)), 2);
    const double oscY = w->grad_amp * w->amp_corr_y * tADC * sinTerm / (double)(nOsc * PI_REF);
    const double oscZ = w->grad_amp * w->amp_corr_z * tADC * sinTerm / (double)(nOsc * PI_REF);

    std::vector<double> gY(gradSamples), gZ(gradSamplesZ);
    for (int i = 0; i < gradSamples; ++i)
        gY[i] = -w->grad_amp * w->amp_corr_y * std::sin(2.0 * PI_REF * nOsc * (double)i / (double)gradSamples);
    for (int i = 0; i < gradSamplesZ; ++i)
        gZ[i] = w->grad_amp * w->amp_corr_z * std::sin(2.0 * PI_REF * (nOsc + 0.5) * (double)i / (double)gradSamplesZ);
    const size_t nY = (size_t)gradSamples * os, nZ = (size_t)gradSamplesZ * os;
    std::vector<double> kY(nY), kZ(nZ);
    kY[0] = 0.0;
    kZ[0] = 0.0;
    for (size_t i = 1; i < nY; ++i) kY[i] = kY[i - 1] + dtOs * 0.5 * (gY[(i - 1) / os] + gY[i / os]);
    for (size_t i = 1; i < nZ; ++i) kZ[i] = kZ[i - 1] + dtOs * 0.5 * (gZ[(i - 1) / os] + gZ[i / os]);

    std::vector<double> hx(sX), hy(sX), hz(sX);
    for (int i = 0; i < sX; ++i) {
        const double tY = (i + 1) * w->dwell - w->shift_y;
        const double tZ = tADC / (4.0 * nOsc) + (i + 1) * w->dwell - w->shift_z;
        long long eY = std::llround(tY / tADC * (double)nY);
        long long eZ = std::llround(tZ / (tADC + 0.5 * tADC / (double)nOsc) * (double)nZ);
        // the reference compares a signed index with size()-1: negatives clamp to the end
        if (eY < 0 || (size_t)eY > nY - 1) eY = (long long)nY - 1;
        if (eZ < 0 || (size_t)eZ > nZ - 1) eZ = (long long)nZ - 1;
        hx[i] = i / (double)(sX - 1.0);
        hy[i] = (tY < 0) ? 0.0 : kY[eY];
        hz[i] = kZ[eZ];
    }
    std::vector<double> traj(3 * (size_t)nSamples);
    double maxY = 0, minY = 0, maxZ = 0, minZ = 0;
    for (long long i = 0; i < nSamples; ++i) {
        const int ix = (int)(i % sX), iy = (int)((i / sX) % sY), iz = (int)(i / ((long long)sX * sY));
        const double by = kmax[1][0] - iy / (double)(sY - 1.0) * (kmax[1][0] - kmax[1][1]);
        const double bz = kmax[2][1] - iz / (double)(sZ - 1.0) * (kmax[2][1] - kmax[2][0]);
        double* t = &traj[3 * (size_t)i];
        t[0] = hx[ix];
        t[1] = by + hy[ix];
        t[2] = bz + hz[ix];
        maxY = std::max(maxY, t[1]);
        minY = std::min(minY, t[1]);
        maxZ = std::max(maxZ, t[2]);
        minZ = std::min(minZ, t[2]);
    }
    const double nBorder = 42.0;
    const double fX = (1.0 * nBorder) / (double)w->gx;
    const double fY = (1.0 * nBorder - 0.405 * oscY / (double)(std::fabs(kmax[1][0]) + std::fabs(kmax[1][1])) * w->gy) / (double)w->gy;
    const double fZ = (1.0 * nBorder - 0.405 * oscZ / (double)(std::fabs(kmax[2][0]) + std::fabs(kmax[2][1])) * w->gz) / (double)w->gz;
    for (long long k = 0; k < nSamples; ++k) {
        double* t = &traj[3 * (size_t)k];
        t[1] -= minY;
        t[2] -= minZ;
        t[1] = t[1] / (double)(maxY - minY);
        t[2] = t[2] / (double)(maxZ - minZ);
        t[0] *= (1.0 - 2 * fX);
        t[1] *= (1.0 - 2 * fY);
        t[2] *= (1.0 - 2 * fZ);
        t[0] += fX;
        t[1] += fY;
        t[2] += fZ;
        const long long i3 = k / ((long long)sX * sY);
        const long long i2 = (k - (long long)sX * sY * i3) / sX;
        const long long i1 = k - (long long)sX * i2 - (long long)sX * sY * i3;
        const long long dst = i3 + (long long)sZ * i2 + (long long)sY * sZ * i1;
        for (int a = 0; a < 3; ++a) k_out[3 * dst + a] = t[a];
    }
    return CGS_OK;
}
