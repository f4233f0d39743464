// Host-side image helpers of the model ingestion path: PNG scanline
// unfiltering (the sequential part of decoding a PNG; chunk parsing and
// inflate stay in the caller).
#include <cstdint>
#include <cstdlib>

#include "api_util.h"

using lucent::clear_error;
using lucent::fail;

namespace {

// Paeth predictor (PNG specification, section 9.4).
inline uint8_t paeth(int a, int b, int c) {
  const int p = a + b - c;
  const int pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
  if (pa <= pb && pa <= pc) return (uint8_t)a;
  return (uint8_t)(pb <= pc ? b : c);
}

}  // namespace

extern "C" lucent_status lucent_png_unfilter(const uint8_t* in, uint32_t rows, uint32_t row_bytes, uint32_t bpp,
                                             uint8_t* out) {
  clear_error();
  if (rows == 0 || row_bytes == 0) return LUCENT_OK;
  if (!in || !out || bpp == 0 || bpp > 8) return fail(LUCENT_ERR_INVALID, "bad PNG unfilter arguments");
  for (uint32_t y = 0; y < rows; y++) {
    const uint8_t* src = in + (size_t)y * (row_bytes + 1);
    const uint8_t type = src[0];
    src++;
    uint8_t* dst = out + (size_t)y * row_bytes;
    const uint8_t* up = y ? dst - row_bytes : nullptr;
    for (uint32_t i = 0; i < row_bytes; i++) {
      const int a = i >= bpp ? dst[i - bpp] : 0;
      const int b = up ? up[i] : 0;
      const int c = (up && i >= bpp) ? up[i - bpp] : 0;
      int v = src[i];
      switch (type) {
        case 0: break;
        case 1: v += a; break;
        case 2: v += b; break;
        case 3: v += (a + b) >> 1; break;
        case 4: v += paeth(a, b, c); break;
        default: return fail(LUCENT_ERR_INVALID, "PNG row %u has filter type %u", y, (unsigned)type);
      }
      dst[i] = (uint8_t)v;
    }
  }
  return LUCENT_OK;
}
