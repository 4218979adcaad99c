// Intensity pyramid and derivative images of the photometric (RGB) term.
//
// Reference: Tracking/Pyrdown.cu (PyrDownGaussKernel<uchar, uchar>
// :201-245, ImageToIntensityKernel :250-260, ComputeDerivativeImageKernel
// :262-304), driven by Frame::FillImages (Core/Frame.cc:74-84).
//
// GB300 form: one launch per level.  Level 0's intensity comes from the
// colour image, each coarser level from the level above; the last launch
// makes every level's derivative images and, beside them, the per-pixel
// flag of the pose-independent half of RGBReduction::FindCorresp (the
// border, the 4x4 window of nonzero intensity and a nonzero gradient), so
// that the per-iteration correspondence pass starts from one byte per
// pixel.  When asked, each level first saves the intensity it overwrites:
// the previous frame's pyramid becomes the last frame's, as SwapFrame
// makes it in the reference.
#include "sf_kernels.cuh"

namespace sf {
namespace {

__constant__ float c_gauss_u8[25] = {1, 4, 6, 4, 1, 4, 16, 24, 16, 4, 6, 24, 36,
                                     24, 6, 4, 16, 24, 16, 4, 1, 4, 6, 4, 1};

__device__ __forceinline__ bool want_save(const int *save_flag) { return save_flag && *save_flag != 0; }

// ImageToIntensityKernel: (int)(0.2125 g + 0.7154 r + 0.0721 b) with the
// double weights, the first byte weighted 0.7154 as written.  The exact
// value is N / 10000 with N = 2125 g + 7154 r + 721 b, at least 1e-4 from
// an integer unless N is a multiple of 10000, while the double expression
// is within 1e-13 of it; so the truncation is N / 10000 except at those
// 1,722 of 2^24 inputs, where the double expression itself decides (it is
// one below N / 10000 at 63 of them).
__global__ void k_intensity(sf_image rgb, sf_image out, sf_image save, const int *save_flag) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= out.cols || y >= out.rows) return;
  const uint8_t *p = row_ptr<const uint8_t>(rgb, y) + 3 * x;
  const int r = p[0], g = p[1], b = p[2];
  const int n = 2125 * g + 7154 * r + 721 * b;
  int v = n / 10000;
  if (v * 10000 == n) v = (int)(0.2125 * (double)g + 0.7154 * (double)r + 0.0721 * (double)b);
  uint8_t *o = row_ptr<uint8_t>(out, y) + x;
  if (want_save(save_flag)) row_ptr<uint8_t>(save, y)[x] = *o;
  *o = (uint8_t)v;
}

// PyrDownGaussKernel<unsigned char, unsigned char>: the reference's
// clipped 5x5 window, reversed tap index and float sums (exact here: every
// sum is an integer below 2^24).
__global__ void k_pyrdown_u8(sf_image src, sf_image dst, sf_image save, const int *save_flag) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= dst.cols || y >= dst.rows) return;
  const int D = 5;
  const int tx = min(2 * x - D / 2 + D, src.cols - 1);
  const int ty = min(2 * y - D / 2 + D, src.rows - 1);
  float sum = 0.f;
  int count = 0;
  for (int cy = max(0, 2 * y - D / 2); cy < ty; ++cy) {
    const uint8_t *row = row_ptr<const uint8_t>(src, cy);
    for (int cx = max(0, 2 * x - D / 2); cx < tx; ++cx) {
      const float k = c_gauss_u8[(ty - cy - 1) * 5 + (tx - cx - 1)];
      sum += (float)row[cx] * k;
      count = (int)((float)count + k);
    }
  }
  uint8_t *o = row_ptr<uint8_t>(dst, y) + x;
  if (want_save(save_flag)) row_ptr<uint8_t>(save, y)[x] = *o;
  *o = (uint8_t)(int)(sum / (float)count);
}

// ComputeDerivativeImageKernel: the Sobel taps run from index 8 down over
// the window clipped to the image (so they shift at the border, as
// written); the float sums are exact integers.  Then the pose-independent
// tests of FindCorresp (Reduction.cu:422-433): 5 <= x < cols - 5,
// 5 <= y < rows - 5, intensity > 0 over rows [y-2, y+2) and columns
// [x-2, x+2), and a nonzero gradient.
struct DerivLevels {
  sf_image img[kMaxLevels], dx[kMaxLevels], dy[kMaxLevels], cand[kMaxLevels];
};

__global__ void k_derivative_cand(DerivLevels a) {
  const int l = blockIdx.z;
  const sf_image im = a.img[l];
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= im.cols || y >= im.rows) return;
  const float sx[9] = {1, 0, -1, 2, 0, -2, 1, 0, -1};
  const float sy[9] = {1, 2, 1, 0, 0, 0, -1, -2, -1};
  float dxv = 0.f, dyv = 0.f;
  int k = 8;
  for (int j = max(y - 1, 0); j <= min(y + 1, im.rows - 1); j++) {
    const uint8_t *row = row_ptr<const uint8_t>(im, j);
    for (int i = max(x - 1, 0); i <= min(x + 1, im.cols - 1); i++) {
      dxv += (float)row[i] * sx[k];
      dyv += (float)row[i] * sy[k];
      --k;
    }
  }
  const short gx = (short)dxv, gy = (short)dyv;
  row_ptr<short>(a.dx[l], y)[x] = gx;
  row_ptr<short>(a.dy[l], y)[x] = gy;
  if (!a.cand[l].data) return;
  bool ok = x >= 5 && x < im.cols - 5 && y >= 5 && y < im.rows - 5 && (gx != 0 || gy != 0);
  if (ok)
    for (int u = y - 2; u < y + 2; ++u) {
      const uint8_t *row = row_ptr<const uint8_t>(im, u);
      for (int v = x - 2; v < x + 2; ++v) ok = ok && row[v] > 0;
    }
  row_ptr<uint8_t>(a.cand[l], y)[x] = ok ? 1 : 0;
}

inline dim3 grid_for(int cols, int rows, dim3 blk, int z = 1) {
  return dim3((cols + blk.x - 1) / blk.x, (rows + blk.y - 1) / blk.y, z);
}

}  // namespace

void launch_intensity(const sf_image &rgb, const sf_image &out, const sf_image *save, const int *save_flag,
                      cudaStream_t s) {
  const dim3 blk(32, 8);
  k_intensity<<<grid_for(out.cols, out.rows, blk), blk, 0, s>>>(rgb, out, save ? *save : sf_image{},
                                                                 save ? save_flag : nullptr);
  note_launch();
}

void launch_pyrdown_u8(const sf_image &src, const sf_image &dst, const sf_image *save, const int *save_flag,
                       cudaStream_t s) {
  const dim3 blk(32, 8);
  k_pyrdown_u8<<<grid_for(dst.cols, dst.rows, blk), blk, 0, s>>>(src, dst, save ? *save : sf_image{},
                                                                  save ? save_flag : nullptr);
  note_launch();
}

void launch_derivatives(const sf_image *img, const sf_image *dx, const sf_image *dy, const sf_image *cand,
                        int levels, cudaStream_t s) {
  DerivLevels a = {};
  for (int l = 0; l < levels; ++l) {
    a.img[l] = img[l];
    a.dx[l] = dx[l];
    a.dy[l] = dy[l];
    a.cand[l] = cand ? cand[l] : sf_image{};
  }
  const dim3 blk(32, 8);
  k_derivative_cand<<<grid_for(img[0].cols, img[0].rows, blk, levels), blk, 0, s>>>(a);
  note_launch();
}

void launch_intensity_pyramid(const sf_image &rgb, const sf_image *img, const sf_image *save,
                              const int *save_flag, const sf_image *dx, const sf_image *dy,
                              const sf_image *cand, int levels, cudaStream_t s) {
  launch_intensity(rgb, img[0], save ? &save[0] : nullptr, save_flag, s);
  for (int l = 1; l < levels; ++l) launch_pyrdown_u8(img[l - 1], img[l], save ? &save[l] : nullptr, save_flag, s);
  launch_derivatives(img, dx, dy, cand, levels, s);
}

}  // namespace sf
