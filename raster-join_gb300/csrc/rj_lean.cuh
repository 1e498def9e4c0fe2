// rj_lean.cuh -- building blocks of the lean label passes (rj_count_kernels.cu,
// rj_lean_kernels.cu): the block-code marker and the pixel arithmetic.
#pragma once
#include "rj_launch.h"

namespace rj {

// Marker in a block-code map: the block's pixels carry different labels.
// 0xFFFD is no polygon label (ids stop at kMaxLabelPolys - 1), nor the empty
// or the hybrid border label.
constexpr uint16_t kCodeMixed = 0xFFFDu;

// Pixel of (x, y) in the tile, equal to pix_of(snap_win(win_coord(...))) of
// the generic pass with fewer operations, by two exact rewrites:
//   * the snap's multiplication by 256 moves into the viewport transform:
//     fl(fl(h*ndc) + h) * 256 == fl(fl(H*ndc) + H) with H = 256 h, since
//     scaling by a power of two commutes with rounding (an h*ndc small enough
//     to be subnormal is absorbed by the addition of h either way);
//   * snap_win clamps the window coordinate to +-2^20 px before converting;
//     here only the lower clamp stays (it also sends NaN below the canvas:
//     fmaxf(NaN, c) = c) and the conversion saturates above, which puts every
//     coordinate beyond the clamp on a pixel outside [0, res) just the same.
// (Packed fp32x2 arithmetic was tried for the two coordinates: each packed
// operation alone rounds like the scalar one, but chains of them did not
// reproduce the scalar results on GB300, so the arithmetic stays scalar.)
struct TileXf2 {
    float sx, tx, Hx;            // per axis: scale, offset, 256 * half resolution
    float sy, ty, Hy;
};

__device__ __forceinline__ TileXf2 tile_xf2(const LabelCountArgs& a) {
    return TileXf2{a.col0.x, a.col0.y, __fmul_rn(a.col0.z, (float)kSub),
                   a.row0.x, a.row0.y, __fmul_rn(a.row0.z, (float)kSub)};
}

__device__ __forceinline__ int snapped_pixel(float v, float s, float t, float H) {
    const float w = __fadd_rn(__fmul_rn(H, __fadd_rn(__fmul_rn(s, v), t)), H);   // window coordinate * 256
    return __float2int_rn(fmaxf(w, -kWinClamp * (float)kSub)) >> kSubpixelBits;
}

// Returns whether the pixel lies in the canvas.
__device__ __forceinline__ bool count_pixel(const LabelCountArgs& a, const TileXf2& xf, float x, float y, int& px,
                                            int& py) {
    px = snapped_pixel(x, xf.sx, xf.tx, xf.Hx);
    py = snapped_pixel(y, xf.sy, xf.ty, xf.Hy);
    return (unsigned)px < (unsigned)a.resx && (unsigned)py < (unsigned)a.resy;
}

}  // namespace rj
