// xb_fits.cpp — FITS primary-HDU reader/writer replacing the reference's
// CCfits calls (src/fitsUtil.cpp:8-64).
//
// Read: BITPIX -32 or -64 (anything else is rejected, as fitsUtil.cpp:20-24
// does), NAXIS1 x NAXIS2 big-endian samples, BSCALE/BZERO applied when
// present, returned as FP64.  Write: BITPIX -32 (FLOAT_IMG,
// fitsUtil.cpp:47), 2880-byte blocks, big-endian.  Byte order is handled
// with shifts, so the code is the same on x86-64 and aarch64.

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

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

uint64_t loadBE(const unsigned char* p, int n) {
  uint64_t v = 0;
  for(int i = 0; i < n; i++) v = (v << 8) | p[i];
  return v;
}

}  // namespace

extern "C" {

int xb_fits_read(const char* path, double** data, int* w, int* h) {
  if(!path || !data || !w || !h) return XB_ERR_ARG;
  *data = nullptr;
  FILE* f = std::fopen(path, "rb");
  if(!f) return XB_ERR_IO;
  std::vector<unsigned char> raw;
  unsigned char blk[2880];
  int bitpix = 0, naxis = -1;
  long n1 = 0, n2 = 0;
  double bscale = 1.0, bzero = 0.0;
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
      else if(cardValue(card, "BITPIX", v)) bitpix = std::atoi(v.c_str());
      else if(cardValue(card, "NAXIS", v)) naxis = std::atoi(v.c_str());
      else if(cardValue(card, "NAXIS1", v)) n1 = std::atol(v.c_str());
      else if(cardValue(card, "NAXIS2", v)) n2 = std::atol(v.c_str());
      else if(cardValue(card, "BSCALE", v)) bscale = std::atof(v.c_str());
      else if(cardValue(card, "BZERO", v)) bzero = std::atof(v.c_str());
    }
  }
  if(bitpix != -32 && bitpix != -64) {
    std::fclose(f);
    return XB_ERR_UNSUPPORTED;
  }
  if(naxis != 2 || n1 <= 0 || n2 <= 0 || n1 > (1L << 20) || n2 > (1L << 20)) {
    std::fclose(f);
    return XB_ERR_UNSUPPORTED;
  }
  const size_t n = (size_t)n1 * (size_t)n2, bytes = n * (size_t)(-bitpix / 8);
  raw.resize(bytes);
  if(std::fread(raw.data(), 1, bytes, f) != bytes) {
    std::fclose(f);
    return XB_ERR_IO;
  }
  std::fclose(f);
  double* out = (double*)std::malloc(n * sizeof(double));
  if(!out) return XB_ERR_NOMEM;
  const bool scaled = bscale != 1.0 || bzero != 0.0;
  for(size_t i = 0; i < n; i++) {
    double v;
    if(bitpix == -32) {
      uint32_t u = (uint32_t)loadBE(&raw[i * 4], 4);
      float fv;
      std::memcpy(&fv, &u, 4);
      v = fv;
    } else {
      uint64_t u = loadBE(&raw[i * 8], 8);
      std::memcpy(&v, &u, 8);
    }
    out[i] = scaled ? bzero + bscale * v : v;
  }
  *data = out;
  *w = (int)n1;
  *h = (int)n2;
  return XB_OK;
}

int xb_fits_write(const char* path, const double* data, int w, int h) {
  if(!path || !data || w <= 0 || h <= 0) return XB_ERR_ARG;
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
  std::vector<unsigned char> out(((n * 4 + 2879) / 2880) * 2880, 0);
  for(size_t i = 0; i < n; i++) {
    float fv = (float)data[i];
    uint32_t u;
    std::memcpy(&u, &fv, 4);
    out[i * 4 + 0] = (unsigned char)(u >> 24);
    out[i * 4 + 1] = (unsigned char)(u >> 16);
    out[i * 4 + 2] = (unsigned char)(u >> 8);
    out[i * 4 + 3] = (unsigned char)u;
  }
  ok = ok && std::fwrite(out.data(), 1, out.size(), f) == out.size();
  ok = (std::fclose(f) == 0) && ok;
  return ok ? XB_OK : XB_ERR_IO;
}

void xb_free(void* p) { std::free(p); }

}  // extern "C"
