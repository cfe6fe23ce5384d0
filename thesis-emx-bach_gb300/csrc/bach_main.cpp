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
//                       (<op>name: sqrt((|target| + |conv|) / gain + 2 rn^2),
//                       the noise model of the stamp chi^2, cd.cl:578)
//   -rn x               read noise (ADU per frame, default 0) of that model,
//                       used by the stamp chi^2 and by -on
//   -gain x             gain (e-/ADU, default 1) of that model
//   -wfit               weight the fit's normal equations by 1 / sigma^2 of
//                       that model (the reference's fit is unweighted)
//   -pk                 evaluate the spatially varying kernel at every pixel
//                       (default: once per kernel-sized block, as the
//                       reference does)
// Output: <op><o> (the convolved image, default diff.fits) and <op>sub.fits.
//
// Many pairs in one process (no counterpart in the reference):
//   BACH -pairs list.txt [-pw n] [-pio n] [-graph] [other flags]
// list.txt holds one pair per line, "template science [prefix]" (paths under
// -ip; '#' starts a comment); pair i writes <op><prefix><o> and
// <op><prefix>sub.fits (default prefix "<i>_").  The pairs stream through
// xb_pipeline: -pio reader and writer threads (default 4) overlap FITS decode
// and encode with -pw GPU workers (default 8); -graph replays frame graphs
// (mixed mode); -im applies to every pair (-om / -on are single-pair only).

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
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
  std::string maskIn, maskOut, noiseOut, pairsFile;
  int pipeWorkers = 8, pipeIo = 4;
  bool graph = false;
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
  if(exists(argc, argv, "-rn")) c.readNoise = c.p.readNoise = std::atof(option(argc, argv, "-rn"));
  if(exists(argc, argv, "-gain")) c.p.gain = std::atof(option(argc, argv, "-gain"));
  c.p.convPerPixel = exists(argc, argv, "-pk") ? 1 : 0;
  c.p.fitWeighted = exists(argc, argv, "-wfit") ? 1 : 0;
  c.p.verbose = c.verbose;
  if(exists(argc, argv, "-pairs")) {
    const char* f = option(argc, argv, "-pairs");
    if(!f) throw std::invalid_argument("-pairs expects a list file");
    c.pairsFile = f;
    if(exists(argc, argv, "-pw")) c.pipeWorkers = std::atoi(option(argc, argv, "-pw"));
    if(exists(argc, argv, "-pio")) c.pipeIo = std::atoi(option(argc, argv, "-pio"));
    c.graph = exists(argc, argv, "-graph");
    return;
  }
  const char* t = option(argc, argv, "-t");
  if(!t) throw std::invalid_argument("Template file Input is required!");
  c.templateName = t;
  const char* s = option(argc, argv, "-s");
  if(!s) throw std::invalid_argument("Science file input is required!");
  c.scienceName = s;
}

// -pairs: every listed pair through one streaming pipeline.
int runPairs(const Cli& cli) {
  std::ifstream in(cli.pairsFile);
  if(!in) {
    std::cout << "Unable to open file '" << cli.pairsFile << "'" << std::endl;
    return 1;
  }
  std::vector<std::string> tp, sp, cp, dp;
  std::string line;
  while(std::getline(in, line)) {
    const size_t hash = line.find('#');
    if(hash != std::string::npos) line.resize(hash);
    std::istringstream ls(line);
    std::string t, s, prefix;
    if(!(ls >> t)) continue;
    if(!(ls >> s)) {
      std::cout << "pair list line without a science image: " << line << std::endl;
      return 1;
    }
    if(!(ls >> prefix)) prefix = std::to_string(tp.size()) + "_";
    tp.push_back(cli.inputPath + "/" + t);
    sp.push_back(cli.inputPath + "/" + s);
    cp.push_back(cli.outPath + prefix + cli.outName);
    dp.push_back(cli.outPath + prefix + "sub.fits");
  }
  const int n = (int)tp.size();
  std::vector<const char*> T(n), S(n), C(n), D(n);
  for(int i = 0; i < n; i++) {
    T[i] = tp[i].c_str();
    S[i] = sp[i].c_str();
    C[i] = cp[i].c_str();
    D[i] = dp[i].c_str();
  }
  xb_pipeline* pl = nullptr;
  int rc = xb_pipeline_create(&cli.p, cli.device, cli.pipeWorkers, cli.pipeIo, &pl);
  if(rc != XB_OK) {
    std::cout << "pipeline creation failed (" << rc << ")" << std::endl;
    return 1;
  }
  std::vector<uint8_t> mask;
  int mw = 0, mh = 0;
  if(!cli.maskIn.empty()) {
    double* M = nullptr;
    const std::string mPath = cli.inputPath + "/" + cli.maskIn;
    if(xb_fits_read(mPath.c_str(), &M, &mw, &mh) != XB_OK) {
      std::cout << "Unable to open file '" << mPath << "'" << std::endl;
      xb_pipeline_destroy(pl);
      return 1;
    }
    mask.resize((size_t)mw * mh);
    for(size_t i = 0; i < mask.size(); i++) mask[i] = M[i] != 0.0 ? 1 : 0;
    xb_free(M);
  }
  for(int i = 0; i < cli.pipeWorkers && rc == XB_OK; i++) {
    xb_ctx* w = nullptr;
    rc = xb_pipeline_worker(pl, i, &w);
    if(rc == XB_OK && cli.graph) rc = xb_set_option(w, "graph", 1);
    if(rc == XB_OK && !mask.empty()) rc = xb_set_input_mask(w, mask.data(), mw, mh);
    if(rc != XB_OK) std::cout << (w ? xb_last_error(w) : "no worker") << std::endl;
  }
  std::vector<int> st(n, XB_OK);
  std::vector<double> ks(n, 0.0);
  if(rc == XB_OK) {
    std::cout << "Running " << n << " pairs..." << std::endl;
    xb_pipeline_run_files(pl, n, T.data(), S.data(), C.data(), D.data(), st.data(), ks.data());
  }
  xb_pipeline_stats ps{};
  xb_pipeline_stats_get(pl, &ps);
  int failed = 0;
  for(int i = 0; i < n && rc == XB_OK; i++) {
    if(st[i] != XB_OK) {
      failed++;
      std::cout << "pair " << i << " (" << tp[i] << ", " << sp[i] << ") failed with status "
                << st[i] << std::endl;
    } else if(cli.verbose) {
      std::cout << "pair " << i << ": kernel sum " << ks[i] << std::endl;
    }
  }
  if(rc == XB_OK)
    std::cout << n - failed << " of " << n << " pairs in " << ps.wall_ms << " ms ("
              << (ps.wall_ms > 0 ? 1000.0 * n / ps.wall_ms : 0.0) << " pairs/s); read "
              << ps.read_ms << " ms, compute " << ps.compute_ms << " ms, write " << ps.write_ms
              << " ms (thread totals)" << std::endl;
  xb_pipeline_destroy(pl);
  return rc == XB_OK && failed == 0 ? 0 : 1;
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
  if(!cli.pairsFile.empty()) return runPairs(cli);
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
  // the mixed path computes on FP32 images: FITS -32 samples convert
  // exactly; anything FP32 cannot hold is refused rather than rounded
  std::vector<float> t32, s32;
  if(cli.p.mode == XB_MODE_MIXED && tw == sw && th == sh) {
    const size_t n = (size_t)tw * th;
    t32.resize(n);
    s32.resize(n);
    bool exact = true;
    for(size_t i = 0; i < n; i++) {
      t32[i] = (float)T[i];
      s32[i] = (float)S[i];
      exact = exact && ((double)t32[i] == T[i] || std::isnan(T[i])) &&
              ((double)s32[i] == S[i] || std::isnan(S[i]));
    }
    if(!exact) {
      std::cout << "mixed mode takes FP32 images; use -mode plain for FP64 data" << std::endl;
      xb_free(T);
      xb_free(S);
      xb_ctx_destroy(ctx);
      return 1;
    }
  }
  rc = t32.empty() ? xb_init(ctx, T, tw, th, S, sw, sh)
                   : xb_init_f32(ctx, t32.data(), tw, th, s32.data(), sw, sh);
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
    const double invGain = cli.p.gain > 0.0 ? 1.0 / cli.p.gain : 1.0;
    for(size_t i = 0; i < img.size(); i++)
      img[i] = std::sqrt((std::fabs(target[i]) + std::fabs(img[i])) * invGain +
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
