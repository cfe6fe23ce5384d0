// bach_main.cpp — the BACH command-line tool over the C ABI.
//
// Same flags, progress messages, output names and "<Stage> took N ms" lines
// as the reference's driver (src/main.cpp:16-159, src/argsUtil.cpp:23-82),
// so tools that parse its output keep working:
//   BACH -t <template> -s <science> [-o name] [-op outprefix] [-ip inpath]
//        [-v] [-vt] [-p n] [-d n] [-sss mp|cl] [-sx n] [-sy n]
// Additional flags (parameters the reference hard-codes, argsUtil.h:33-53):
//   -mode plain|mixed   precision mode (default plain)
//   -ko n  -bo n        spatial kernel order / background order
//   -kw n  -ssw n       half kernel width / half substamp width
//   -th x  -tl x        threshHigh / threshLow
//   -gauss s:d,s:d,...  Gaussian sigmas and polynomial degrees
//   -im file            input mask (FITS, <ip>/file; nonzero pixels are
//                       excluded: INPUT_MASK | BAD_INPUT before the dilation)
//   -om name            also write the final mask (<op>name, the 13 flag bits
//                       as FITS values)
//   -on name            also write the noise image of the difference
//                       (<op>name: sqrt(|target| + |conv| + 2 rn^2), gain 1,
//                       the noise model of the reference's chi^2, cd.cl:578)
//   -rn x               read noise for -on (ADU, default 0)
// Output: <op><o> (the convolved image, default diff.fits) and <op>sub.fits.

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "xbach.h"

namespace {

using Clock = std::chrono::steady_clock;

long msBetween(Clock::time_point a, Clock::time_point b) {
  return (long)std::chrono::duration_cast<std::chrono::milliseconds>(b - a).count();
}

const char* option(int argc, const char** argv, const std::string& o) {
  for(int i = 1; i < argc; i++)
    if(o == argv[i]) return i + 1 < argc ? argv[i + 1] : nullptr;
  return nullptr;
}
bool exists(int argc, const char** argv, const std::string& o) {
  for(int i = 1; i < argc; i++)
    if(o == argv[i]) return true;
  return false;
}

struct Cli {
  std::string templateName, scienceName, outName = "diff.fits", inputPath = "res/",
                                         outPath = "out/";
  std::string maskIn, maskOut, noiseOut;
  double readNoise = 0.0;
  bool verbose = false, verboseTime = false;
  int device = 0;
  xb_params p{};
};

void parse(int argc, const char** argv, Cli& c) {
  xb_params_default(&c.p);
  if(exists(argc, argv, "-o")) c.outName = option(argc, argv, "-o");
  if(exists(argc, argv, "-op")) c.outPath = option(argc, argv, "-op");
  if(exists(argc, argv, "-ip")) c.inputPath = option(argc, argv, "-ip");
  if(exists(argc, argv, "-sx")) c.p.stampsx = std::atoi(option(argc, argv, "-sx"));
  if(exists(argc, argv, "-sy")) c.p.stampsy = std::atoi(option(argc, argv, "-sy"));
  if(exists(argc, argv, "-sss")) {
    std::string m = option(argc, argv, "-sss");
    if(m != "mp" && m != "cl") throw std::invalid_argument("sss mode should be mp or cl");
  }
  c.verbose = exists(argc, argv, "-v");
  c.verboseTime = exists(argc, argv, "-vt");
  if(exists(argc, argv, "-d")) c.device = std::atoi(option(argc, argv, "-d"));
  if(exists(argc, argv, "-mode")) {
    std::string m = option(argc, argv, "-mode");
    if(m == "plain") c.p.mode = XB_MODE_PLAIN;
    else if(m == "mixed") c.p.mode = XB_MODE_MIXED;
    else throw std::invalid_argument("mode should be plain or mixed");
  }
  if(exists(argc, argv, "-ko")) c.p.kernelOrder = std::atoi(option(argc, argv, "-ko"));
  if(exists(argc, argv, "-bo")) c.p.backgroundOrder = std::atoi(option(argc, argv, "-bo"));
  if(exists(argc, argv, "-kw")) c.p.hKernelWidth = std::atoi(option(argc, argv, "-kw"));
  if(exists(argc, argv, "-ssw")) c.p.hSStampWidth = std::atoi(option(argc, argv, "-ssw"));
  if(exists(argc, argv, "-th")) c.p.threshHigh = std::atof(option(argc, argv, "-th"));
  if(exists(argc, argv, "-tl")) c.p.threshLow = std::atof(option(argc, argv, "-tl"));
  if(exists(argc, argv, "-gauss")) {
    std::stringstream ss(option(argc, argv, "-gauss"));
    std::string item;
    int n = 0;
    while(std::getline(ss, item, ',') && n < XB_MAX_GAUSS) {
      double sigma = 0;
      int deg = 0;
      if(std::sscanf(item.c_str(), "%lf:%d", &sigma, &deg) != 2 || sigma <= 0)
        throw std::invalid_argument("-gauss expects sigma:degree,...");
      c.p.bg[n] = (float)(1.0 / (2.0 * sigma * sigma));
      c.p.dg[n] = deg;
      n++;
    }
    c.p.nGauss = n;
  }
  if(exists(argc, argv, "-im")) c.maskIn = option(argc, argv, "-im");
  if(exists(argc, argv, "-om")) c.maskOut = option(argc, argv, "-om");
  if(exists(argc, argv, "-on")) c.noiseOut = option(argc, argv, "-on");
  if(exists(argc, argv, "-rn")) c.readNoise = std::atof(option(argc, argv, "-rn"));
  c.p.verbose = c.verbose;
  const char* t = option(argc, argv, "-t");
  if(!t) throw std::invalid_argument("Template file Input is required!");
  c.templateName = t;
  const char* s = option(argc, argv, "-s");
  if(!s) throw std::invalid_argument("Science file input is required!");
  c.scienceName = s;
}

int fail(xb_ctx* ctx, int rc) {
  std::cout << (ctx ? xb_last_error(ctx) : "error") << std::endl;
  if(ctx) xb_ctx_destroy(ctx);
  return rc == XB_OK ? 0 : 1;
}

}  // namespace

int main(int argc, const char* argv[]) {
  const auto p1 = Clock::now();
  Cli cli;
  try {
    std::cout << "Reading in arguments..." << std::endl;
    parse(argc, argv, cli);
  } catch(const std::invalid_argument& e) {
    std::cout << e.what() << '\n';
    return 1;
  }
  std::cout << "\nReading in images..." << std::endl;
  if(cli.verbose)
    std::cout << "template image name: " << cli.templateName
              << ", science image name: " << cli.scienceName << std::endl;
  double *T = nullptr, *S = nullptr;
  int tw = 0, th = 0, sw = 0, sh = 0;
  const std::string tPath = cli.inputPath + "/" + cli.templateName;
  const std::string sPath = cli.inputPath + "/" + cli.scienceName;
  if(xb_fits_read(tPath.c_str(), &T, &tw, &th) != XB_OK) {
    std::cout << "Unable to open file '" << tPath << "'" << std::endl;
    return 1;
  }
  if(xb_fits_read(sPath.c_str(), &S, &sw, &sh) != XB_OK) {
    std::cout << "Unable to open file '" << sPath << "'" << std::endl;
    xb_free(T);
    return 1;
  }
  std::cout << "\nSetting up CUDA..." << std::endl;
  xb_ctx* ctx = nullptr;
  int rc = xb_ctx_create(&cli.p, cli.device, &ctx);
  if(rc != XB_OK) {
    std::cout << "context creation failed (" << rc << ")" << std::endl;
    return 1;
  }
  if(!cli.maskIn.empty()) {
    double* M = nullptr;
    int mw = 0, mh = 0;
    const std::string mPath = cli.inputPath + "/" + cli.maskIn;
    if(xb_fits_read(mPath.c_str(), &M, &mw, &mh) != XB_OK) {
      std::cout << "Unable to open file '" << mPath << "'" << std::endl;
      xb_free(T);
      xb_free(S);
      xb_ctx_destroy(ctx);
      return 1;
    }
    std::vector<uint8_t> m((size_t)mw * mh);
    for(size_t i = 0; i < m.size(); i++) m[i] = M[i] != 0.0 ? 1 : 0;
    xb_free(M);
    rc = xb_set_input_mask(ctx, m.data(), mw, mh);
    if(rc != XB_OK) {
      xb_free(T);
      xb_free(S);
      return fail(ctx, rc);
    }
  }
  rc = xb_init(ctx, T, tw, th, S, sw, sh);
  // the noise image needs the target frame after the fit
  std::vector<double> tCopy, sCopy;
  if(rc == XB_OK && !cli.noiseOut.empty()) {
    tCopy.assign(T, T + (size_t)tw * th);
    sCopy.assign(S, S + (size_t)sw * sh);
  }
  xb_free(T);
  xb_free(S);
  if(rc != XB_OK) return fail(ctx, rc);
  auto p2 = Clock::now();
  if(cli.verboseTime) std::cout << "Ini took " << msBetween(p1, p2) << " ms" << std::endl;

  auto p3 = Clock::now();
  std::cout << "\nCreating stamps..." << std::endl;
  std::cout << "Identifying sub-stamps..." << std::endl;
  if((rc = xb_sss(ctx)) != XB_OK) return fail(ctx, rc);
  if(cli.verbose) {
    double n0 = 0, n1 = 0;
    xb_get_scalar(ctx, "nstamps0", &n0);
    xb_get_scalar(ctx, "nstamps1", &n1);
    std::cout << "Non-Empty template stamps: " << n0 << std::endl;
    std::cout << "Non-Empty science stamps: " << n1 << std::endl;
  }
  auto p4 = Clock::now();
  if(cli.verboseTime) std::cout << "SSS took " << msBetween(p3, p4) << " ms" << std::endl;
  std::cout << std::endl;

  auto p5 = Clock::now();
  std::cout << "\nCalculating matrix variables..." << std::endl;
  if((rc = xb_cmv(ctx)) != XB_OK) return fail(ctx, rc);
  auto p6 = Clock::now();
  if(cli.verboseTime) std::cout << "CMV took " << msBetween(p5, p6) << " ms" << std::endl;

  auto p7 = Clock::now();
  std::cout << "\nChoosing convolution direction..." << std::endl;
  int convTemplate = 0;
  if((rc = xb_cd(ctx, &convTemplate)) != XB_OK) return fail(ctx, rc);
  double m0 = 0, m1 = 0;
  xb_get_scalar(ctx, "merit0", &m0);
  xb_get_scalar(ctx, "merit1", &m1);
  std::cout << "template merit value = " << m0 << ", science merit value = " << m1 << std::endl;
  if(cli.verbose)
    std::cout << (convTemplate ? cli.templateName : cli.scienceName) << " chosen to be convolved."
              << std::endl;
  auto p8 = Clock::now();
  if(cli.verboseTime) std::cout << "CD took " << msBetween(p7, p8) << " ms" << std::endl;

  auto p9 = Clock::now();
  std::cout << "\nFitting kernel..." << std::endl;
  if((rc = xb_ksc(ctx)) != XB_OK) return fail(ctx, rc);
  auto p10 = Clock::now();
  if(cli.verboseTime) std::cout << "KSC took " << msBetween(p9, p10) << " ms" << std::endl;

  auto p11 = Clock::now();
  std::cout << "\nConvolving..." << std::endl;
  double kernSum = 0;
  if((rc = xb_conv(ctx, &kernSum)) != XB_OK) return fail(ctx, rc);
  if(cli.verbose)
    std::cout << "Sum of kernel at (" << tw / 2 << "," << th / 2 << "): " << kernSum << std::endl;
  auto p12 = Clock::now();
  if(cli.verboseTime) std::cout << "Conv took " << msBetween(p11, p12) << " ms" << std::endl;

  auto p13 = Clock::now();
  std::cout << "\nSubtracting images..." << std::endl;
  if((rc = xb_sub(ctx)) != XB_OK) return fail(ctx, rc);
  auto p14 = Clock::now();
  if(cli.verboseTime) std::cout << "Sub took " << msBetween(p13, p14) << " ms" << std::endl;

  auto p15 = Clock::now();
  std::cout << "\nWriting output..." << std::endl;
  std::vector<double> img((size_t)tw * th);
  const std::string convPath = cli.outPath + cli.outName, subPath = cli.outPath + "sub.fits";
  if((rc = xb_get_image_f64(ctx, XB_IMG_CONV, img.data())) != XB_OK) return fail(ctx, rc);
  if(xb_fits_write(convPath.c_str(), img.data(), tw, th) != XB_OK) {
    std::cout << "Unable to save file '" << convPath << "'" << std::endl;
    xb_ctx_destroy(ctx);
    return 1;
  }
  if((rc = xb_get_image_f64(ctx, XB_IMG_DIFF, img.data())) != XB_OK) return fail(ctx, rc);
  if(xb_fits_write(subPath.c_str(), img.data(), tw, th) != XB_OK) {
    std::cout << "Unable to save file '" << subPath << "'" << std::endl;
    xb_ctx_destroy(ctx);
    return 1;
  }
  if(!cli.maskOut.empty()) {
    std::vector<uint16_t> m((size_t)tw * th);
    if((rc = xb_get_mask(ctx, m.data())) != XB_OK) return fail(ctx, rc);
    for(size_t i = 0; i < m.size(); i++) img[i] = m[i];
    const std::string path = cli.outPath + cli.maskOut;
    if(xb_fits_write(path.c_str(), img.data(), tw, th) != XB_OK) {
      std::cout << "Unable to save file '" << path << "'" << std::endl;
      xb_ctx_destroy(ctx);
      return 1;
    }
  }
  if(!cli.noiseOut.empty()) {
    if((rc = xb_get_image_f64(ctx, XB_IMG_CONV, img.data())) != XB_OK) return fail(ctx, rc);
    const std::vector<double>& target = convTemplate ? sCopy : tCopy;
    for(size_t i = 0; i < img.size(); i++)
      img[i] = std::sqrt(std::fabs(target[i]) + std::fabs(img[i]) +
                         2.0 * cli.readNoise * cli.readNoise);
    const std::string path = cli.outPath + cli.noiseOut;
    if(xb_fits_write(path.c_str(), img.data(), tw, th) != XB_OK) {
      std::cout << "Unable to save file '" << path << "'" << std::endl;
      xb_ctx_destroy(ctx);
      return 1;
    }
  }
  auto p16 = Clock::now();
  if(cli.verboseTime) std::cout << "Fin took " << msBetween(p15, p16) << " ms" << std::endl;
  std::cout << "omp time " << msBetween(p1, p16) / 1000.0 << std::endl;
  std::cout << "\nBACH finished." << std::endl;
  if(cli.verboseTime) std::cout << "BACH took " << msBetween(p1, p16) << " ms" << std::endl;
  xb_ctx_destroy(ctx);
  return 0;
}
