// gridding_common.cuh -- tap-record helpers shared by the gridding kernels:
// the packed nearest grid point and the 64-byte record load.
#pragma once
#include "cgs_common.cuh"
#include "cgs_types.h"

namespace cgs {

CGS_D unsigned pack_nearest(int nx, int ny, int nz)
{
    return (unsigned)nx | ((unsigned)ny << 11) | ((unsigned)nz << 22);
}
CGS_D void unpack_nearest(unsigned u, int& nx, int& ny, int& nz)
{
    nx = (int)(u & 2047u);
    ny = (int)((u >> 11) & 2047u);
    nz = (int)(u >> 22);
}


CGS_D void load_record(const TapRecord* __restrict__ rec, long long i, float (&w)[15], int& nx, int& ny,
                       int& nz)
{
    const float4* p = reinterpret_cast<const float4*>(rec + i);
    const float4 a = __ldg(p + 0), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3);
    w[0] = a.x; w[1] = a.y; w[2] = a.z; w[3] = a.w;
    w[4] = b.x; w[5] = b.y; w[6] = b.z; w[7] = b.w;
    w[8] = c.x; w[9] = c.y; w[10] = c.z; w[11] = c.w;
    w[12] = d.x; w[13] = d.y; w[14] = d.z;
    unpack_nearest(__float_as_uint(d.w), nx, ny, nz);
}

}  // namespace cgs
