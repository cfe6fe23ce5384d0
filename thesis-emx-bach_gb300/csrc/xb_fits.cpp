// xb_fits.cpp — FITS primary-HDU reader/writer replacing the reference's
// CCfits calls (src/fitsUtil.cpp:8-64).
//
// Read: BITPIX -32 or -64 (anything else is rejected, as fitsUtil.cpp:20-24
// does), NAXIS1 x NAXIS2 big-endian samples, BSCALE/BZERO applied when
// present, returned as FP64.  Write: BITPIX -32 (FLOAT_IMG,
// fitsUtil.cpp:47), 2880-byte blocks, big-endian.  Byte order is handled
// with shifts, so the code is the same on x86-64 and aarch64.  The helpers in
// namespace xb (xb_fits.h) also decode unscaled BITPIX -32 samples straight
// into FP32 buffers, for the streaming pipeline.

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <algorithm>
#include <vector>

#include "xb_fits.h"
#include "xbach.h"

namespace {

bool cardValue(const char* card, const char* key, std::string& val) {
  size_t kl = std::strlen(key);
  if(std::strncmp(card, key, kl) != 0) return false;
  for(size_t i = kl; i < 8; i++)
    if(card[i] != ' ') return false;
  if(card[8] != '=') return false;
  std::string v(card + 10, 70);
  size_t slash = v.find('/');
  if(slash != std::string::npos && v.find('\'') == std::string::npos) v = v.substr(0, slash);
  size_t a = v.find_first_not_of(' '), b = v.find_last_not_of(' ');
  val = a == std::string::npos ? "" : v.substr(a, b - a + 1);
  return true;
}

inline uint32_t loadBE32(const unsigned char* p) {
  return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | (uint32_t)p[3];
}
inline uint64_t loadBE64(const unsigned char* p) {
  return (uint64_t)loadBE32(p) << 32 | loadBE32(p + 4);
}
inline void storeBE32(unsigned char* p, uint32_t u) {
  p[0] = (unsigned char)(u >> 24);
  p[1] = (unsigned char)(u >> 16);
  p[2] = (unsigned char)(u >> 8);
  p[3] = (unsigned char)u;
}

constexpr size_t CHUNK = 1 << 16;  // samples converted per fread / fwrite

}  // namespace

namespace xb {

int fitsOpen(const char* path, FitsHeader& hd, FILE** fp) {
  *fp = nullptr;
  FILE* f = std::fopen(path, "rb");
  if(!f) return XB_ERR_IO;
  unsigned char blk[2880];
  int naxis = -1;
  long n1 = 0, n2 = 0;
  hd = FitsHeader{};
  bool end = false;
  while(!end) {
    if(std::fread(blk, 1, 2880, f) != 2880) {
      std::fclose(f);
      return XB_ERR_IO;
    }
    for(int c = 0; c < 36 && !end; c++) {
      const char* card = (const char*)blk + 80 * c;
      std::string v;
      if(std::strncmp(card, "END     ", 8) == 0) end = true;
      else if(cardValue(card, "BITPIX", v)) hd.bitpix = std::atoi(v.c_str());
      else if(cardValue(card, "NAXIS", v)) naxis = std::atoi(v.c_str());
      else if(cardValue(card, "NAXIS1", v)) n1 = std::atol(v.c_str());
      else if(cardValue(card, "NAXIS2", v)) n2 = std::atol(v.c_str());
      else if(cardValue(card, "BSCALE", v)) hd.bscale = std::atof(v.c_str());
      else if(cardValue(card, "BZERO", v)) hd.bzero = std::atof(v.c_str());
    }
  }
  // BITPIX -32 / -64 only, as src/fitsUtil.cpp:20-24 accepts
  if((hd.bitpix != -32 && hd.bitpix != -64) || naxis != 2 || n1 <= 0 || n2 <= 0 ||
     n1 > (1L << 20) || n2 > (1L << 20)) {
    std::fclose(f);
    return XB_ERR_UNSUPPORTED;
  }
  hd.w = (int)n1;
  hd.h = (int)n2;
  *fp = f;
  return XB_OK;
}

int fitsReadSamples(FILE* f, const FitsHeader& hd, void* dst, bool asDouble) {
  const size_t n = (size_t)hd.w * hd.h, sz = (size_t)(-hd.bitpix / 8);
  if(!asDouble && !hd.exactF32()) return XB_ERR_UNSUPPORTED;
  if((sz == 4) == !asDouble) {
    // same width: read in place, then swap in place
    unsigned char* b = (unsigned char*)dst;
    if(std::fread(b, sz, n, f) != n) return XB_ERR_IO;
    if(sz == 4) {
      for(size_t i = 0; i < n; i++) {
        const uint32_t u = loadBE32(b + 4 * i);
        std::memcpy(b + 4 * i, &u, 4);
      }
    } else {
      for(size_t i = 0; i < n; i++) {
        const uint64_t u = loadBE64(b + 8 * i);
        std::memcpy(b + 8 * i, &u, 8);
      }
    }
  } else {
    // FP32 samples widened to FP64, through a chunk buffer
    std::vector<unsigned char> raw(CHUNK * 4);
    double* out = (double*)dst;
    for(size_t i0 = 0; i0 < n; i0 += CHUNK) {
      const size_t m = std::min(CHUNK, n - i0);
      if(std::fread(raw.data(), 4, m, f) != m) return XB_ERR_IO;
      for(size_t i = 0; i < m; i++) {
        const uint32_t u = loadBE32(&raw[4 * i]);
        float fv;
        std::memcpy(&fv, &u, 4);
        out[i0 + i] = fv;
      }
    }
  }
  if(asDouble && hd.scaled()) {
    double* out = (double*)dst;
    for(size_t i = 0; i < n; i++) out[i] = hd.bzero + hd.bscale * out[i];
  }
  return XB_OK;
}

int fitsWrite(const char* path, const float* f32, const double* f64, int w, int h) {
  // the reference writes to "!" + path: overwrite an existing file
  FILE* f = std::fopen(path, "wb");
  if(!f) return XB_ERR_IO;
  std::string hdr;
  auto card = [&](const std::string& s) {
    std::string c = s;
    c.resize(80, ' ');
    hdr += c;
  };
  char buf[96];
  card("SIMPLE  =                    T / file does conform to FITS standard");
  card("BITPIX  =                  -32 / number of bits per data pixel");
  card("NAXIS   =                    2 / number of data axes");
  std::snprintf(buf, sizeof buf, "NAXIS1  = %20d / length of data axis 1", w);
  card(buf);
  std::snprintf(buf, sizeof buf, "NAXIS2  = %20d / length of data axis 2", h);
  card(buf);
  card("EXTEND  =                    T / FITS dataset may contain extensions");
  card("END");
  hdr.resize((hdr.size() + 2879) / 2880 * 2880, ' ');
  bool ok = std::fwrite(hdr.data(), 1, hdr.size(), f) == hdr.size();
  const size_t n = (size_t)w * h;
  std::vector<unsigned char> out(CHUNK * 4);
  for(size_t i0 = 0; ok && i0 < n; i0 += CHUNK) {
    const size_t m = std::min(CHUNK, n - i0);
    for(size_t i = 0; i < m; i++) {
      const float fv = f32 ? f32[i0 + i] : (float)f64[i0 + i];
      uint32_t u;
      std::memcpy(&u, &fv, 4);
      storeBE32(&out[4 * i], u);
    }
    ok = std::fwrite(out.data(), 4, m, f) == m;
  }
  const size_t pad = (2880 - (n * 4) % 2880) % 2880;
  if(ok && pad) {
    std::memset(out.data(), 0, pad);
    ok = std::fwrite(out.data(), 1, pad, f) == pad;
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? XB_OK : XB_ERR_IO;
}

}  // namespace xb

extern "C" {

int xb_fits_read(const char* path, double** data, int* w, int* h) {
  if(!path || !data || !w || !h) return XB_ERR_ARG;
  *data = nullptr;
  xb::FitsHeader hd;
  FILE* f = nullptr;
  int rc = xb::fitsOpen(path, hd, &f);
  if(rc != XB_OK) return rc;
  double* out = (double*)std::malloc((size_t)hd.w * hd.h * sizeof(double));
  if(!out) {
    std::fclose(f);
    return XB_ERR_NOMEM;
  }
  rc = xb::fitsReadSamples(f, hd, out, true);
  std::fclose(f);
  if(rc != XB_OK) {
    std::free(out);
    return rc;
  }
  *data = out;
  *w = hd.w;
  *h = hd.h;
  return XB_OK;
}

int xb_fits_write(const char* path, const double* data, int w, int h) {
  if(!path || !data || w <= 0 || h <= 0) return XB_ERR_ARG;
  return xb::fitsWrite(path, nullptr, data, w, h);
}

void xb_free(void* p) { std::free(p); }

}  // extern "C"
