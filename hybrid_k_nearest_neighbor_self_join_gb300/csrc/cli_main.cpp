// cli_main.cpp -- `main <FNAME> <DIM> <K>`, the reference's command line
// (main.cu:109-510) on the GB300 library.
//
// Same arguments and messages as the reference: a wrong argument count or a
// DIM that differs from a fixed GPUNUMDIM build prints the reference's text
// and exits 0 (main.cu:123-146).  The dataset is read with importNDDataset's
// CSV rules, the join runs on the GPU, and the verification checksum line of
// main.cu:452 is printed.  The params.h switches PRINTNEIGHBORTABLE and
// PRINTOUTLIERSCORES (params.h:20-22) are read from the environment
// (KNNSJ_PRINTNEIGHBORTABLE, KNNSJ_PRINTOUTLIERSCORES; default 0) or fixed
// with -D at build time; when set, KNN_out.txt / KNN_out_distances.txt /
// KNN_outlier_scores.txt are written to the working directory.  One line per
// run is appended to gpu_stats.txt, as main.cu:472-489 does.  A FNAME ending
// in .npy, .bin or .raw is read as binary (NumPy array or raw values of the
// build's DTYPE) instead of CSV.

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/knnsj.h"

#ifndef KNNSJ_BUILD_DTYPE_DOUBLE
typedef float dtype_t;
static const knnsj_dtype kDtype = KNNSJ_F32;
static const char* kDtypeName = "float";
#else
typedef double dtype_t;
static const knnsj_dtype kDtype = KNNSJ_F64;
static const char* kDtypeName = "double";
#endif

static int env_flag(const char* name, int dflt) {
  const char* v = std::getenv(name);
  return (v && *v) ? std::atoi(v) : dflt;
}

int main(int argc, char* argv[]) {
  if (argc != 4) {
    std::printf("\n\nIncorrect number of input parameters.  \nShould be dataset file, number of dimensions, kNN\n");
    return 0;
  }
  const char* fname = argv[1];
  const unsigned int NDIM = (unsigned int)std::atoi(argv[2]);
  const unsigned int kNN = (unsigned int)std::atoi(argv[3]);
#ifdef GPUNUMDIM
  if (GPUNUMDIM != NDIM) {
    std::printf(
        "\nERROR: The number of dimensions defined for the GPU is not the same as the number of dimensions\n \
		 passed into the computer program on the command line. GPUNUMDIM=%d, NDIM=%d Exiting!!!",
        GPUNUMDIM, NDIM);
    return 0;
  }
#endif
  if (NDIM == 0) {
    std::fprintf(stderr, "knnsj: DIM must be positive\n");
    return 1;
  }
  // FNAME ending in .npy, .bin or .raw is read as binary (knnsj_read_binary),
  // anything else as the reference's CSV
  auto ends_with = [&](const char* suf) {
    const size_t a = std::strlen(fname), b = std::strlen(suf);
    return a >= b && std::strcmp(fname + a - b, suf) == 0;
  };
  const bool binary = ends_with(".npy") || ends_with(".bin") || ends_with(".raw");
  auto read = [&](void* out, uint64_t* cnt) {
    return binary ? knnsj_read_binary(fname, kDtype, NDIM, out, cnt) : knnsj_read_csv(fname, kDtype, NDIM, out, cnt);
  };
  uint64_t n = 0;
  knnsj_status s = read(nullptr, &n);
  if (s != KNNSJ_OK) {
    std::fprintf(stderr, "knnsj: cannot read %s: %s\n", fname, knnsj_status_string(s));
    return 1;
  }
  std::vector<dtype_t> data((size_t)n * NDIM);
  s = read(data.data(), &n);
  if (s != KNNSJ_OK) {
    std::fprintf(stderr, "knnsj: cannot read %s: %s\n", fname, knnsj_status_string(s));
    return 1;
  }
  std::printf("\nNumber of data points: %llu", (unsigned long long)n);
  const uint64_t K = (uint64_t)kNN + 1;
  std::vector<int32_t> ids((size_t)(n * K), -1);
  std::vector<dtype_t> dists((size_t)(n * K), 0);
  knnsj_options o;
  std::memset(&o, 0, sizeof(o));
  o.struct_size = sizeof(o);
  o.beta = -1.0;
  o.device = -1;
#ifdef NUMINDEXEDDIM
  o.num_indexed_dims = NUMINDEXEDDIM;
#endif
#ifdef BETA
  o.beta = BETA;
#endif
  knnsj_stats st;
  std::memset(&st, 0, sizeof(st));
  st.struct_size = sizeof(st);
  const auto t0 = std::chrono::steady_clock::now();
  s = knnsj_selfjoin(data.data(), kDtype, n, NDIM, kNN, &o, ids.data(), dists.data(), &st);
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (s != KNNSJ_OK) {
    std::fprintf(stderr, "knnsj: join failed: %s\n", knnsj_status_string(s));
    return 1;
  }
  std::printf("\nMain: estimate of epsilon: %0.9f", st.eps0);
  std::printf("\nTime to join only: %f", secs);
  std::printf("\n[Verification] Total distance (without square root): %f", st.total_distance);
#ifndef PRINTNEIGHBORTABLE
#define PRINTNEIGHBORTABLE 0
#endif
#ifndef PRINTOUTLIERSCORES
#define PRINTOUTLIERSCORES 0
#endif
  if (env_flag("KNNSJ_PRINTNEIGHBORTABLE", PRINTNEIGHBORTABLE)) {
    s = knnsj_write_knn_out(".", n, (uint32_t)K, ids.data(), dists.data(), kDtype);
    if (s != KNNSJ_OK) std::fprintf(stderr, "knnsj: cannot write KNN_out.txt\n");
  }
  if (env_flag("KNNSJ_PRINTOUTLIERSCORES", PRINTOUTLIERSCORES)) {
    s = knnsj_write_outlier_scores(".", n, (uint32_t)K, ids.data(), dists.data(), kDtype);
    if (s != KNNSJ_OK) std::fprintf(stderr, "knnsj: cannot write KNN_outlier_scores.txt\n");
  }
  if (FILE* f = std::fopen("gpu_stats.txt", "a")) {
    std::fprintf(f,
                 "%f, %s, KNN: %u, Eps bucket: %d, Total dist: %.9g, "
                 "GPUNUMDIM/NUMINDEXEDDIM/BETA/DTYPE(float/double): %u, %d, %g, %s\n",
                 secs, fname, kNN, st.eps_bucket, st.total_distance, NDIM, o.num_indexed_dims, o.beta,
                 kDtypeName);
    std::fclose(f);
  }
  std::printf("\n\n");
  return 0;
}
