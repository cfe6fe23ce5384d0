// xb_fits.h — FITS primary-HDU helpers shared by the public reader/writer
// (xb_fits_read / xb_fits_write) and the streaming pipeline, which decodes
// into and encodes from its own pinned buffers.
#pragma once

#include <cstddef>
#include <cstdio>

namespace xb {

struct FitsHeader {
  int w = 0, h = 0;
  int bitpix = 0;             // -32 or -64 (anything else is rejected)
  double bscale = 1.0, bzero = 0.0;
  bool scaled() const { return bscale != 1.0 || bzero != 0.0; }
  // samples that FP32 holds exactly: unscaled BITPIX -32
  bool exactF32() const { return bitpix == -32 && !scaled(); }
};

// Opens path and parses the primary header; on XB_OK *f is positioned at the
// first sample (the caller closes it).  Status codes of include/xbach.h.
int fitsOpen(const char* path, FitsHeader& hd, FILE** f);

// Reads the w*h samples after fitsOpen into dst: FP32 when hd.exactF32() and
// asDouble is false, else FP64 with BSCALE/BZERO applied.  dst holds
// w*h*(asDouble ? 8 : 4) bytes.
int fitsReadSamples(FILE* f, const FitsHeader& hd, void* dst, bool asDouble);

// Writes a BITPIX -32 primary HDU (big-endian, 2880-byte blocks) from FP32
// (f32 != nullptr) or FP64 samples rounded to FP32.
int fitsWrite(const char* path, const float* f32, const double* f64, int w, int h);

}  // namespace xb
