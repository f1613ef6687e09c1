// Plain-form correlation: the double launch configurations (the kernel is in
// piv_corr_fft.cuh).
#include "piv_corr_fft.cuh"

namespace piv {

static const FftVariant kFft8d[] = {PIV_FFT_VAR(8, double, 1, 8, 16, 128)};
static const FftVariant kFft16d[] = {PIV_FFT_VAR(16, double, 1, 16, 8, 128), PIV_FFT_VAR(16, double, 4, 4, 8, 128)};
static const FftVariant kFft32d[] = {PIV_FFT_VAR(32, double, 4, 8, 4, 128), PIV_FFT_VAR(32, double, 8, 4, 4, 128),
                                     PIV_FFT_VAR(32, double, 4, 8, 2, 128)};
static const FftVariant kFft64d[] = {PIV_FFT_VAR(64, double, 8, 8, 1, 256), PIV_FFT_VAR(64, double, 4, 16, 1, 256),
                                     PIV_FFT_VAR(64, double, 8, 8, 1, 512)};
static const FftVariant kFft128d[] = {PIV_FFT_VAR(128, double, 8, 16, 1, 512),
                                      PIV_FFT_VAR(128, double, 16, 8, 1, 512)};
static const FftVariant kFft256d[] = {PIV_FFT_VAR(256, double, 16, 16, 1, 1024)};

const FftVariant* fft_variants_f64(int fft_size, int* count) {
  *count = 0;
  switch (fft_size) {
    case 8: return table(kFft8d, count);
    case 16: return table(kFft16d, count);
    case 32: return table(kFft32d, count);
    case 64: return table(kFft64d, count);
    case 128: return table(kFft128d, count);
    case 256: return table(kFft256d, count);
    default: return nullptr;
  }
}

}  // namespace piv
