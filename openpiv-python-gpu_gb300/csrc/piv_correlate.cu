// Plain-form correlation: the float launch configurations, the variant
// tables' dispatch and the entry points (the kernel is in piv_corr_fft.cuh).
#include <algorithm>

#include "piv_corr_fft.cuh"

namespace piv {

static const FftVariant kFft8f[] = {PIV_FFT_VAR(8, float, 1, 8, 16, 128), PIV_FFT_VAR(8, float, 1, 8, 32, 256),
                                    PIV_FFT_VAR(8, float, 2, 4, 16, 128)};
static const FftVariant kFft16f[] = {PIV_FFT_VAR(16, float, 1, 16, 8, 128), PIV_FFT_VAR(16, float, 1, 16, 16, 256),
                                     PIV_FFT_VAR(16, float, 4, 4, 8, 128), PIV_FFT_VAR(16, float, 1, 16, 4, 64)};
static const FftVariant kFft32f[] = {PIV_FFT_VAR(32, float, 1, 32, 4, 128), PIV_FFT_VAR(32, float, 4, 8, 4, 128),
                                     PIV_FFT_VAR(32, float, 8, 4, 4, 128), PIV_FFT_VAR(32, float, 1, 32, 8, 256),
                                     PIV_FFT_VAR(32, float, 4, 8, 8, 256), PIV_FFT_VAR(32, float, 1, 32, 2, 64)};
// The defaults of N = 64 and 128 are the fastest variants measured on the
// 1024 x 1024 three-pass workload; they share the radix split of the next
// entry, so their results are the same bit for bit.
static const FftVariant kFft64f[] = {PIV_FFT_VAR(64, float, 8, 8, 1, 128), PIV_FFT_VAR(64, float, 8, 8, 1, 256),
                                     PIV_FFT_VAR(64, float, 4, 16, 1, 256), PIV_FFT_VAR(64, float, 16, 4, 1, 256),
                                     PIV_FFT_VAR(64, float, 8, 8, 2, 256), PIV_FFT_VAR(64, float, 8, 8, 2, 512)};
static const FftVariant kFft128f[] = {PIV_FFT_VAR(128, float, 8, 16, 1, 1024), PIV_FFT_VAR(128, float, 8, 16, 1, 512),
                                      PIV_FFT_VAR(128, float, 16, 8, 1, 512), PIV_FFT_VAR(128, float, 8, 16, 1, 256),
                                      PIV_FFT_VAR(128, float, 4, 32, 1, 512)};
static const FftVariant kFft256f[] = {PIV_FFT_VAR(256, float, 16, 16, 1, 1024)};

const FftVariant* fft_variants_f64(int fft_size, int* count);  // piv_correlate_f64.cu

static const FftVariant* fft_variants(int fft_size, int dtype, int* count) {
  *count = 0;
  if (dtype == PIV_DTYPE_F64) return fft_variants_f64(fft_size, count);
  switch (fft_size) {
    case 8: return table(kFft8f, count);
    case 16: return table(kFft16f, count);
    case 32: return table(kFft32f, count);
    case 64: return table(kFft64f, count);
    case 128: return table(kFft128f, count);
    case 256: return table(kFft256f, count);
    default: return nullptr;
  }
}

int correlate_fft_variant_count(int fft_size, int dtype) {
  int n = 0;
  fft_variants(fft_size, dtype, &n);
  return n;
}

int correlate_fft_variant_describe(int fft_size, int dtype, int variant, int* r1, int* r2, int* wpc, int* nt) {
  int n = 0;
  const FftVariant* t = fft_variants(fft_size, dtype, &n);
  if (!t || variant < 0 || variant >= n) return PIV_E_ARG;
  *r1 = t[variant].r1;
  *r2 = t[variant].r2;
  *wpc = t[variant].wpc;
  *nt = t[variant].nt;
  return PIV_OK;
}

size_t correlate_fft_scratch_bytes(int fft_size, int dtype) {
  int n = 0;
  const FftVariant* t = fft_variants(fft_size, dtype, &n);
  size_t need = 0;
  for (int k = 0; k < n; ++k) need = std::max(need, t[k].scratch());
  return need;
}

int correlate_fft(const CorrArgs& a, int variant, cudaStream_t stream) {
  int n = 0;
  const FftVariant* t = fft_variants(a.fft_size, a.dtype, &n);
  if (!t) return set_error(PIV_E_UNSUPPORTED, "fft_size %d is not supported (8..256)", a.fft_size);
  if (variant < 0 || variant >= n) variant = 0;
  return t[variant].launch(a, stream);
}

}  // namespace piv
