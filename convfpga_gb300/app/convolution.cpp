// convolution: command-line driver of the GB300 FFT convolution library, with the
// flags and flow of pc2/ConvFPGA's sample application (src/main.cpp, src/helper.cpp):
//
//   -p/--path F        plan-cache file passed to fpga_initialize (required unless -c)
//   -w/--wisdomfile F  accepted for compatibility (FFTW wisdom; no FFTW here)
//   -n/--num N         cube size (default 64)          -i/--iter K   iterations (1)
//   -t/--threads T     CPU threads for -c / verify (1)  -b/--batch B  signals (1)
//   -y/--noverify      skip the CPU check               -c/--cpu-only CPU path only
//   -s/--usesvm        SVM entry points                  -e/--emulate  emulation platform name
//   -a/--autotune      time the plan variants for N and write them to the plan-cache file
//                      (-p) before running: the analogue of building FFTW wisdom
//
// Flow as src/main.cpp:11-106: initialise, allocate with fpgaf_complex_malloc, fill with
// rand()/RAND_MAX, run the entry point the flags select (fpgaf_conv3D, fpgaf_conv3D_svm,
// fpgaf_conv3D_svm_batch; a non-SVM batch, which the reference rejects, runs through
// convgpu_conv3d_host), check each iteration against a CPU convolution with the
// reference's criterion (SNR > 120 dB, src/fft_conv3D.cpp:236-258) and report the
// mean and deviation of the fpga_t timings (src/helper.cpp:180-275). Unlike the
// reference app, every batch slot gets its own signal (src/helper.cpp:159-171 copies
// signal 0 to hide a batch bug the library no longer has).
//
// The CPU convolution (verification and -c) is this program's own double-precision
// radix-2 FFT on T threads: the reference uses FFTW, which is not available.
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "convgpu.h"

namespace {

struct Config {
  std::string path;
  std::string wisdomfile = "a.out";
  unsigned num = 64, iter = 1, threads = 1, batch = 1;
  bool noverify = false, cpuonly = false, usesvm = false, emulate = false, autotune = false;
};

void usage() {
  std::printf(
      "convolution - 3D FFT-based convolution on the GPU\n"
      "  -p, --path F        plan-cache file (required unless --cpu-only)\n"
      "  -w, --wisdomfile F  accepted, unused (no FFTW)\n"
      "  -n, --num N         cube size, power of two 16..512 (default 64)\n"
      "  -i, --iter K        iterations (default 1)\n"
      "  -t, --threads T     CPU threads (default 1)\n"
      "  -y, --noverify      no CPU verification\n"
      "  -b, --batch B       signals per call (default 1)\n"
      "  -c, --cpu-only      CPU convolution only\n"
      "  -s, --usesvm        SVM entry points\n"
      "  -e, --emulate       emulation platform name\n"
      "  -a, --autotune      tune the plan for N and write it to the plan-cache file\n"
      "  -h, --help          this text\n");
}

bool parse(int argc, char **argv, Config &c) {
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    auto val = [&](const char *name) -> const char * {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "Error parsing options: %s needs a value\n", name);
        std::exit(1);
      }
      return argv[++i];
    };
    if (a == "-h" || a == "--help") {
      usage();
      std::exit(0);
    } else if (a == "-p" || a == "--path") c.path = val("path");
    else if (a == "-w" || a == "--wisdomfile") c.wisdomfile = val("wisdomfile");
    else if (a == "-n" || a == "--num") c.num = (unsigned)std::strtoul(val("num"), nullptr, 10);
    else if (a == "-i" || a == "--iter") c.iter = (unsigned)std::strtoul(val("iter"), nullptr, 10);
    else if (a == "-t" || a == "--threads") c.threads = (unsigned)std::strtoul(val("threads"), nullptr, 10);
    else if (a == "-b" || a == "--batch") c.batch = (unsigned)std::strtoul(val("batch"), nullptr, 10);
    else if (a == "-y" || a == "--noverify") c.noverify = true;
    else if (a == "-c" || a == "--cpu-only") c.cpuonly = true;
    else if (a == "-s" || a == "--usesvm") c.usesvm = true;
    else if (a == "-e" || a == "--emulate") c.emulate = true;
    else if (a == "-a" || a == "--autotune") c.autotune = true;
    else {
      std::fprintf(stderr, "Error parsing options: unknown option %s\n", a.c_str());
      return false;
    }
  }
  if (c.iter == 0 || c.threads == 0 || c.batch == 0) {
    std::fprintf(stderr, "Error parsing options: iter, threads and batch must be positive\n");
    return false;
  }
  if (!c.cpuonly && c.path.empty()) {
    std::printf("\tPlease input path to bitstream\n");
    std::exit(1);
  }
  return true;
}

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ---------------------------------------------------------------- CPU convolution (double)
using cd = std::complex<double>;

// In-place radix-2 decimation-in-time FFT of one strided pencil; sign -1 forward,
// +1 unnormalised backward.
void fft1d(cd *base, size_t stride, unsigned n, int sign, const std::vector<cd> &tw, std::vector<cd> &tmp) {
  for (unsigned i = 0; i < n; ++i) tmp[i] = base[i * stride];
  for (unsigned i = 1, j = 0; i < n; ++i) {  // bit-reversal permutation
    unsigned bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(tmp[i], tmp[j]);
  }
  for (unsigned len = 2; len <= n; len <<= 1) {
    const unsigned step = n / len;
    for (unsigned i = 0; i < n; i += len)
      for (unsigned k = 0; k < len / 2; ++k) {
        cd w = tw[k * step];
        if (sign > 0) w = std::conj(w);
        const cd u = tmp[i + k], v = tmp[i + k + len / 2] * w;
        tmp[i + k] = u + v;
        tmp[i + k + len / 2] = u - v;
      }
  }
  for (unsigned i = 0; i < n; ++i) base[i * stride] = tmp[i];
}

void fft3d(cd *vol, unsigned n, int sign, unsigned threads) {
  std::vector<cd> tw(n / 2);
  for (unsigned k = 0; k < n / 2; ++k) tw[k] = std::polar(1.0, -2.0 * M_PI * k / n);
  const size_t nn = (size_t)n * n;
  for (int axis = 0; axis < 3; ++axis) {
    auto work = [&](unsigned t0) {
      std::vector<cd> tmp(n);
      for (size_t p = t0; p < nn; p += threads) {
        const size_t a = p / n, b = p % n;  // the two coordinates that fix the pencil
        if (axis == 0) fft1d(vol + p * n, 1, n, sign, tw, tmp);
        else if (axis == 1) fft1d(vol + a * nn + b, n, n, sign, tw, tmp);
        else fft1d(vol + p, nn, n, sign, tw, tmp);
      }
    };
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < threads; ++t) pool.emplace_back(work, t);
    work(0);
    for (auto &th : pool) th.join();
  }
}

// out[b] = IFFT3(FFT3(sig[b]) * FFT3(filter)), unnormalised, in double precision.
void cpu_conv(unsigned n, const float2 *sig, const float2 *filter, unsigned batch, std::vector<cd> &out,
              unsigned threads, double *filter_ms, double *conv_ms) {
  const size_t pts = (size_t)n * n * n;
  std::vector<cd> f(pts);
  for (size_t i = 0; i < pts; ++i) f[i] = cd(filter[i].x, filter[i].y);
  double t0 = now_ms();
  fft3d(f.data(), n, -1, threads);
  if (filter_ms) *filter_ms = now_ms() - t0;
  out.assign(pts * batch, cd());
  t0 = now_ms();
  for (unsigned b = 0; b < batch; ++b) {
    cd *v = out.data() + b * pts;
    for (size_t i = 0; i < pts; ++i) v[i] = cd(sig[b * pts + i].x, sig[b * pts + i].y);
    fft3d(v, n, -1, threads);
    for (size_t i = 0; i < pts; ++i) v[i] *= f[i];
    fft3d(v, n, +1, threads);
  }
  if (conv_ms) *conv_ms = (now_ms() - t0) / batch;
}

double snr_db(const std::vector<cd> &ref, const float2 *out) {
  double mag = 0, noise = 0;
  for (size_t i = 0; i < ref.size(); ++i) {
    const double dr = ref[i].real() - out[i].x, di = ref[i].imag() - out[i].y;
    mag += std::norm(ref[i]);
    noise += dr * dr + di * di;
  }
  return noise == 0 ? INFINITY : 10.0 * std::log10(mag / noise);
}

void create_data(float2 *inp, size_t pts) {
  for (size_t j = 0; j < pts; ++j) {
    inp[j].x = (float)rand() / (float)RAND_MAX;
    inp[j].y = (float)rand() / (float)RAND_MAX;
  }
}

void report(const Config &c, const std::vector<fpga_t> &rt) {
  auto field = [&](double fpga_t::*m, double &mean, double &sd) {
    mean = 0;
    for (auto &r : rt) mean += r.*m;
    mean /= rt.size();
    double var = 0;
    for (auto &r : rt) var += (r.*m - mean) * (r.*m - mean);
    sd = std::sqrt(var / rt.size());
  };
  double fw, fws, fe, fes, sw, sws, se, ses, si, sis, sr, srs;
  field(&fpga_t::filter_pcie_wr_t, fw, fws);
  field(&fpga_t::filter_exec_t, fe, fes);
  field(&fpga_t::sig_pcie_wr_t, sw, sws);
  field(&fpga_t::sig_exec_t, se, ses);
  field(&fpga_t::siginv_exec_t, si, sis);
  field(&fpga_t::sig_pcie_rd_t, sr, srs);
  std::printf("\n\n------------------------------------------\nMeasurements in ms\n");
  std::printf("--------------------------------------------\n%s", c.iter > 1 ? "Average Measurements of iterations\n" : "");
  std::printf("GPU:\n-----\n- Filter:\n");
  std::printf("  Host to Device      : %g\n  Execution           : %g\n\n", fw, fe);
  std::printf("- Signal Convolution:\n  Host to Device      : %g\n", sw);
  std::printf("  FFT + Conv          : %g\n  Inverse FFT         : %g\n", se, si);
  std::printf("  Total Computation   : %g\n", se + si);
  if (c.batch > 1) std::printf("  Total Comp per batch: %g\n", (se + si) / c.batch);
  std::printf("  Device to Host      : %g\n", sr);
  if (c.iter > 1) {
    std::printf("\nDeviation of runtimes among iterations\n- Filter:\n");
    std::printf("Host to Dev         = %.4lfms\nExecution           = %.4lfms\n", fws, fes);
    std::printf("- Signal:\nFFT + Conv          = %.4lfms\nInverse FFT         = %.4lfms\n", ses, sis);
    std::printf("Total Computation   = %.4lfms\n", ses + sis);
    std::printf("Host to Dev         = %.4lfms\nDev to Host         = %.4lfms\n\n", sws, srs);
  }
}

}  // namespace

int main(int argc, char **argv) {
  Config c;
  if (!parse(argc, argv, c)) return EXIT_FAILURE;
  std::printf("\nCONFIGURATION: \n---------------\n");
  std::printf("Plan cache   = %s\nPoints       = {%u, %u, %u}\nThreads      = %u\n", c.path.c_str(), c.num, c.num,
              c.num, c.threads);
  std::printf("Iterations   = %u\nBatch        = %u\n----------------\n\n", c.iter, c.batch);
  if (c.num < 16 || c.num > 512 || (c.num & (c.num - 1))) {
    std::fprintf(stderr, "num must be a power of two in 16..512\n");
    return EXIT_FAILURE;
  }
  const size_t pts = (size_t)c.num * c.num * c.num;
  if (c.cpuonly) {
    std::vector<float2> f(pts), s(pts);
    create_data(f.data(), pts);
    create_data(s.data(), pts);
    double filt_ms = 0, conv_sum = 0;
    std::vector<cd> out;
    for (unsigned it = 0; it < c.iter; ++it) {
      double fm = 0, cm = 0;
      cpu_conv(c.num, s.data(), f.data(), 1, out, c.threads, &fm, &cm);
      if (it == 0) filt_ms = fm;
      conv_sum += cm;
    }
    std::printf("\n\nMEASUREMENTS \n--------------\nPoints           : %u^3\nThreads          : %u\n", c.num, c.threads);
    std::printf("Iterations       : %u\n\nCPU:\n----\nFilter Runtime   : %gms\n", c.iter, filt_ms);
    std::printf("Conv3D Runtime   : %gms\n\n", conv_sum / c.iter);
    return EXIT_SUCCESS;
  }
  const char *platform = c.emulate ? "Intel(R) FPGA Emulation Platform for OpenCL(TM)" : "Intel(R) FPGA SDK for OpenCL(TM)";
  if (fpga_initialize(platform, c.path.c_str(), c.usesvm) != 0) {
    std::fprintf(stderr, "FPGA initialization error\n");
    return EXIT_FAILURE;
  }
  if (c.autotune) {
    const unsigned sizes[1] = {c.num};
    if (convgpu_autotune(sizes, 1, 1) != 0) {
      std::fprintf(stderr, "autotune error: %s\n", convgpu_last_error());
      return EXIT_FAILURE;
    }
    std::printf("Plan for %u^3 tuned and written to %s\n", c.num, c.path.c_str());
  }
  float2 *filter = (float2 *)fpgaf_complex_malloc(sizeof(float2) * pts);
  float2 *sig = (float2 *)fpgaf_complex_malloc(sizeof(float2) * pts * c.batch);
  float2 *out = (float2 *)fpgaf_complex_malloc(sizeof(float2) * pts * c.batch);
  std::vector<fpga_t> runtime(c.iter);
  int rc = EXIT_SUCCESS;
  create_data(filter, pts);
  create_data(sig, pts * c.batch);
  std::vector<cd> ref;
  if (!c.noverify) cpu_conv(c.num, sig, filter, c.batch, ref, c.threads, nullptr, nullptr);
  for (unsigned i = 0; i < c.iter && rc == EXIT_SUCCESS; ++i) {
    std::printf("\n%u: Calculating Conv3D\n", i);
    if (c.usesvm && c.batch > 1) runtime[i] = fpgaf_conv3D_svm_batch(c.num, sig, filter, out, c.batch);
    else if (c.usesvm) runtime[i] = fpgaf_conv3D_svm(c.num, sig, filter, out);
    else if (c.batch > 1) runtime[i] = convgpu_conv3d_host(c.num, sig, filter, out, c.batch, 0);
    else runtime[i] = fpgaf_conv3D(c.num, sig, filter, out);
    if (!runtime[i].valid) {
      std::fprintf(stderr, "FPGA execution found invalid: %s\n", convgpu_last_error());
      rc = EXIT_FAILURE;
      break;
    }
    if (!c.noverify) {
      const double db = snr_db(ref, out);
      if (db > 120.0) {
        std::printf("Iter %u: verified, SNR %.1f dB\n", i, db);
      } else {
        std::printf("Signal to noise ratio on output sample: %g --> FAILED\n\n", db);
        std::fprintf(stderr, "Iter %u: FPGA result incorrect in comparison to CPU\n", i);
        rc = EXIT_FAILURE;
      }
    }
  }
  fpga_final();
  if (rc == EXIT_SUCCESS) report(c, runtime);
  std::free(sig);
  std::free(filter);
  std::free(out);
  return rc;
}
