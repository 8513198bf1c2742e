// Host launchers of the plane kernels (xy_plane.cuh), compiled in their own
// translation unit.  combo = 100 VX + VY for FFT domains Px = 32 VX, Py = 16 VY.
#pragma once
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace mvr {

// The plane-kernel shape for an FP32 FFT domain P (x, y), or 0 when none exists.
int xy_combo(const int P[3]);
// The pair-kernel shape (two CTAs per plane, a thread-block cluster) for P, or 0.  Shape codes
// >= 10000 select the pair kernels in every launcher below.
int xy_pair_combo(const int P[3]);
// Statistics partials per block written by an update launch over `planes` planes.
int xy_partial_slots(int combo, int planes);
size_t xy_smem(int combo);

// The forward and quotient passes walk the (block, plane) items with one CTA per SM
// (persist, unless MVR_XY_PERSIST=0) or take one CTA per plane; the update pass takes one
// CTA per plane (grid Pz x nb).  Every call returns the launch status.
cudaError_t xy_fwd_mirror(int combo, const float *psi, float2 *S, const BlockMaps &bms, int nb, int Pz, long long Pc,
                          const float2 *twx, const float2 *twy, cudaStream_t s, bool persist = true);
cudaError_t xy_fwd_zero(int combo, const float *blk, float2 *S, const BlockMaps &bms, int nb, int Pz, long long Pc,
                        const float2 *twx, const float2 *twy, cudaStream_t s, bool persist = true);
cudaError_t xy_fwd_kernel(int combo, const SrcKernel &src, float2 *S, const BlockMaps &bms, int nb, int Pz,
                          long long Pc, const float2 *twx, const float2 *twy, cudaStream_t s, bool persist = true);
// the quotient pass over the planes [z0, z0 + nzb) of each block
cudaError_t xy_ratio(int combo, float2 *S, const float *img, const BlockMaps &bms, int nb, int z0, int nzb,
                     long long Pc, const float2 *twx, const float2 *twy, cudaStream_t s, bool persist = true);
cudaError_t xy_update(int combo, int epi, float2 *S, const UpdateArgs &ua, const BlockMaps &bms, int nb, int Pz,
                      long long Pc, const float2 *twx, const float2 *twy, cudaStream_t s);

}  // namespace mvr
