// hostio.cpp -- host-only pieces of the C ABI: dimension order, grid
// dimensions, CSV import, KNN_out text output and outlier scores.
// None of these touches the GPU.

#include <algorithm>
#include <cerrno>
#include <clocale>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <locale.h>
#include <string>
#include <vector>

#include <omp.h>

#include "knnsj_host.h"

using namespace knnsj;

namespace {

// ---- CSV (import_dataset.cpp:50-106) --------------------------------------
//
// The reference reads comma-separated fields with getline(in, f, ',') and
// extracts numbers from each field with `stringstream >> DTYPE` until one
// fails.  libstdc++'s extraction skips whitespace, gathers
// [sign] digits [. digits] [e|E [sign] digits] (the exponent only after a
// mantissa digit), converts the gathered text with strtof / strtod in the
// "C" locale, and fails when nothing was gathered, when the text is not fully
// converted (e.g. "1e+"), or when the value overflows.  Fields are
// independent, so they are parsed in parallel and concatenated in order.

locale_t c_locale() {
  static locale_t loc = newlocale(LC_ALL_MASK, "C", (locale_t)0);
  return loc;
}

inline bool is_ws(char c) { return c == ' ' || c == '\n' || c == '\r' || c == '\t' || c == '\v' || c == '\f'; }
inline bool is_digit(char c) { return c >= '0' && c <= '9'; }

// Extracts one number from [p, end); returns false when extraction fails.
template <typename T>
bool extract_number(const char*& p, const char* end, T* out) {
  while (p < end && is_ws(*p)) p++;
  if (p >= end) return false;
  char buf[128];
  size_t n = 0;
  const char* q = p;
  auto put = [&](char c) {
    if (n < sizeof(buf) - 1) buf[n++] = c;
  };
  if (q < end && (*q == '+' || *q == '-')) put(*q++);
  bool mant = false, dot = false;
  while (q < end) {
    if (is_digit(*q)) {
      mant = true;
      put(*q++);
    } else if (*q == '.' && !dot) {
      dot = true;
      put(*q++);
    } else {
      break;
    }
  }
  if (mant && q < end && (*q == 'e' || *q == 'E')) {
    put(*q++);
    if (q < end && (*q == '+' || *q == '-')) put(*q++);
    while (q < end && is_digit(*q)) put(*q++);
  }
  p = q;
  buf[n] = '\0';
  if (n == 0) return false;
  char* stop = nullptr;
  errno = 0;
  T v;
  if (sizeof(T) == 4)
    v = (T)strtof_l(buf, &stop, c_locale());
  else
    v = (T)strtod_l(buf, &stop, c_locale());
  if (stop == buf || *stop != '\0') return false;
  if (std::isinf(v)) return false;
  *out = v;
  return true;
}

template <typename T>
knnsj_status read_csv_impl(const char* path, uint32_t d, T* out, uint64_t* n_points) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return KNNSJ_ERR_IO;
  std::fseek(f, 0, SEEK_END);
  const long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  std::vector<char> text((size_t)std::max(sz, 0L));
  if (sz > 0 && std::fread(text.data(), 1, (size_t)sz, f) != (size_t)sz) {
    std::fclose(f);
    return KNNSJ_ERR_IO;
  }
  std::fclose(f);
  const char* base = text.data();
  const size_t len = text.size();
  const int nt = std::max(1, std::min(omp_get_max_threads(), (int)(len / (1 << 20)) + 1));
  std::vector<size_t> cut(nt + 1, len);
  cut[0] = 0;
  for (int t = 1; t < nt; t++) {
    size_t c = len * t / nt;
    while (c < len && base[c] != ',') c++;
    cut[t] = c < len ? c + 1 : len;  // each chunk starts right after a comma
    if (cut[t] < cut[t - 1]) cut[t] = cut[t - 1];
  }
  std::vector<std::vector<T>> parts(nt);
#pragma omp parallel for num_threads(nt) schedule(static, 1)
  for (int t = 0; t < nt; t++) {
    const char* p = base + cut[t];
    const char* stop = base + cut[t + 1];
    std::vector<T>& v = parts[t];
    while (p < stop) {
      const char* fend = (const char*)std::memchr(p, ',', (size_t)(stop - p));
      if (!fend) fend = stop;
      const char* q = p;
      T x;
      while (extract_number<T>(q, fend, &x)) v.push_back(x);
      p = fend < stop ? fend + 1 : stop;
    }
  }
  uint64_t total = 0;
  for (auto& v : parts) total += v.size();
  const uint64_t npts = total / d;
  *n_points = npts;
  if (!out) return KNNSJ_OK;
  uint64_t at = 0;
  for (auto& v : parts) {
    const uint64_t take = std::min<uint64_t>(v.size(), npts * d - std::min<uint64_t>(at, npts * d));
    std::memcpy(out + at, v.data(), take * sizeof(T));
    at += take;
  }
  return KNNSJ_OK;
}

// ---- printNeighborTable (main.cu:911-949) ---------------------------------
// std::ostream's default float output is printf("%g") of the value widened to
// double; ids print as plain integers; every entry is followed by ", ".
template <typename T>
knnsj_status write_knn_out_impl(const char* dir, uint64_t n, uint32_t K, const int32_t* ids,
                                const T* dists) {
  const std::string d = dir ? dir : ".";
  const std::string names[2] = {d + "/KNN_out.txt", d + "/KNN_out_distances.txt"};
  const char* headers[2] = {"#data point (line is the point id), neighbor point ids\n",
                            "#data point (line is the point id), neighbor point distances\n"};
  for (int which = 0; which < 2; which++) {
    FILE* f = std::fopen(names[which].c_str(), "wb");
    if (!f) return KNNSJ_ERR_IO;
    std::fputs(headers[which], f);
    const uint64_t chunk = 1 << 16;
    const uint64_t nchunks = (n + chunk - 1) / chunk;
    std::vector<std::string> out(omp_get_max_threads());
    for (uint64_t c0 = 0; c0 < nchunks; c0 += out.size()) {
      const uint64_t c1 = std::min<uint64_t>(nchunks, c0 + out.size());
#pragma omp parallel for schedule(static, 1)
      for (int64_t c = (int64_t)c0; c < (int64_t)c1; c++) {
        std::string& s = out[c - c0];
        s.clear();
        char tmp[64];
        for (uint64_t i = (uint64_t)c * chunk; i < std::min<uint64_t>(n, (uint64_t)(c + 1) * chunk); i++) {
          for (uint32_t j = 0; j < K; j++) {
            int m;
            if (which == 0)
              m = std::snprintf(tmp, sizeof(tmp), "%d, ", ids[i * K + j]);
            else
              m = std::snprintf(tmp, sizeof(tmp), "%g, ", (double)dists[i * K + j]);
            s.append(tmp, (size_t)m);
          }
          s.push_back('\n');
        }
      }
      for (uint64_t c = c0; c < c1; c++) std::fwrite(out[c - c0].data(), 1, out[c - c0].size(), f);
    }
    if (std::fclose(f) != 0) return KNNSJ_ERR_IO;
  }
  return KNNSJ_OK;
}

// ---- printOutlierScores (main.cu:952-1067) --------------------------------
// Same element types and std::sort comparators as the reference
// (compareByPointValue main.cu:62-65, compareByPointFrequencyInOtherSets
// main.cu:68-71), so equal scores are ranked exactly as there.  Ids outside
// [0, n) (unfilled rows) are not counted.
template <typename T>
struct PointDist {
  int pointID;
  T distance;
};
struct PointFreq {
  int pointID;
  uint64_t numTimesInOtherSet;
};

template <typename T>
knnsj_status write_outlier_impl(const char* dir, uint64_t n, uint32_t K, const int32_t* ids, const T* dists) {
  std::vector<T> total(n);
  std::vector<PointDist<T>> kv(n);
  for (uint64_t i = 0; i < n; i++) {
    T t = 0;
    for (uint32_t j = 0; j < K; j++) t += dists[i * K + j];
    total[i] = t;
    kv[i].pointID = (int)i;
    kv[i].distance = t;
  }
  std::sort(kv.begin(), kv.end(),
            [](const PointDist<T>& a, const PointDist<T>& b) { return a.distance > b.distance; });
  std::vector<int> rank1(n);
  for (uint64_t i = 0; i < n; i++) rank1[kv[i].pointID] = (int)i;
  std::vector<PointFreq> fq(n);
  std::vector<uint64_t> indeg(n, 0);
  for (uint64_t i = 0; i < n; i++) {
    fq[i].pointID = (int)i;
    fq[i].numTimesInOtherSet = 0;
  }
  for (uint64_t i = 0; i < n; i++)
    for (uint32_t j = 0; j < K; j++) {
      const int32_t idx = ids[i * K + j];
      if (idx < 0 || (uint64_t)idx >= n) continue;
      fq[idx].numTimesInOtherSet++;
      indeg[idx]++;
    }
  std::sort(fq.begin(), fq.end(),
            [](const PointFreq& a, const PointFreq& b) { return a.numTimesInOtherSet < b.numTimesInOtherSet; });
  std::vector<unsigned int> rank2(n);
  for (uint64_t i = 0; i < n; i++) rank2[fq[i].pointID] = (unsigned int)i;
  const std::string path = std::string(dir ? dir : ".") + "/KNN_outlier_scores.txt";
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return KNNSJ_ERR_IO;
  std::fputs(
      "#data point (line is the point id), col0: mean distance between point and its k neighbors,"
      "col1: outlier ranking for col0, col2: the number of times the point appears in another set "
      "(in-degree), col3: the ranking for col2 \n",
      f);
  for (uint64_t i = 0; i < n; i++) {
    const double mean = total[i] / ((K * 1.0) - 1.0);
    std::fprintf(f, "%g, %d, %llu, %u\n", mean, rank1[i], (unsigned long long)indeg[i], rank2[i]);
  }
  if (std::fclose(f) != 0) return KNNSJ_ERR_IO;
  return KNNSJ_OK;
}

// ---- binary input: NumPy .npy (format 1.0-3.0) or raw little-endian values ---
// Neither exists in the reference, which reads CSV only
// (import_dataset.cpp:50-106); at tens of millions of points a binary file
// is read in a fraction of the time the text parse takes.
struct BinLayout {
  uint64_t offset = 0;   // first data byte
  uint64_t values = 0;   // values in the file
  int elem = 0;          // 4 (float32) or 8 (float64)
  bool ok = false;
};

// Parses the .npy header (magic, version, header length, the dict with
// 'descr', 'fortran_order' and 'shape'); raw files are taken as values of
// the requested type.  Big-endian and Fortran-ordered arrays are refused.
BinLayout bin_layout(FILE* f, uint64_t fsize, int want_elem) {
  BinLayout L;
  unsigned char head[10];
  const size_t got = std::fread(head, 1, sizeof(head), f);
  if (got >= 10 && head[0] == 0x93 && std::memcmp(head + 1, "NUMPY", 5) == 0) {
    const int major = head[6];
    uint64_t hlen = 0, pre = 0;
    if (major == 1) {
      hlen = (uint64_t)head[8] | ((uint64_t)head[9] << 8);
      pre = 10;
    } else if (major == 2 || major == 3) {
      unsigned char b[2];
      if (std::fread(b, 1, 2, f) != 2) return L;
      hlen = (uint64_t)head[8] | ((uint64_t)head[9] << 8) | ((uint64_t)b[0] << 16) | ((uint64_t)b[1] << 24);
      pre = 12;
    } else {
      return L;
    }
    if (hlen > (1u << 20) || pre + hlen > fsize) return L;
    std::string h(hlen, '\0');
    if (std::fseek(f, (long)pre, SEEK_SET) != 0 || std::fread(&h[0], 1, hlen, f) != hlen) return L;
    const size_t dp = h.find("'descr'");
    if (dp == std::string::npos) return L;
    const size_t q1 = h.find('\'', h.find(':', dp) + 1);
    const size_t q2 = q1 == std::string::npos ? q1 : h.find('\'', q1 + 1);
    if (q2 == std::string::npos) return L;
    const std::string descr = h.substr(q1 + 1, q2 - q1 - 1);
    if (descr == "<f4" || descr == "=f4" || descr == "f4")
      L.elem = 4;
    else if (descr == "<f8" || descr == "=f8" || descr == "f8")
      L.elem = 8;
    else
      return L;
    const size_t fo = h.find("'fortran_order'");
    if (fo == std::string::npos || h.find("True", fo) < h.find(',', fo)) return L;
    const size_t sp = h.find("'shape'");
    if (sp == std::string::npos) return L;
    const size_t p1 = h.find('(', sp), p2 = h.find(')', sp);
    if (p1 == std::string::npos || p2 == std::string::npos) return L;
    uint64_t count = 1;
    const std::string dims = h.substr(p1 + 1, p2 - p1 - 1);
    size_t i = 0;
    bool any = false;
    while (i < dims.size()) {
      while (i < dims.size() && (dims[i] == ' ' || dims[i] == ',')) i++;
      if (i >= dims.size()) break;
      char* end = nullptr;
      const unsigned long long v = std::strtoull(dims.c_str() + i, &end, 10);
      if (end == dims.c_str() + i) return L;
      count *= v;
      any = true;
      i = (size_t)(end - dims.c_str());
    }
    if (!any) count = 1;  // a 0-d array holds one value
    L.offset = pre + hlen;
    L.values = count;
    if (L.offset + count * (uint64_t)L.elem > fsize) return L;
    L.ok = true;
    return L;
  }
  L.offset = 0;
  L.elem = want_elem;
  L.values = fsize / (uint64_t)want_elem;
  L.ok = fsize % (uint64_t)want_elem == 0;
  return L;
}

template <typename T>
knnsj_status read_binary_impl(const char* path, uint32_t d, T* out, uint64_t* n_points) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return KNNSJ_ERR_IO;
  std::fseek(f, 0, SEEK_END);
  const long fs = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (fs < 0) {
    std::fclose(f);
    return KNNSJ_ERR_IO;
  }
  const BinLayout L = bin_layout(f, (uint64_t)fs, (int)sizeof(T));
  std::fclose(f);
  if (!L.ok) return KNNSJ_ERR_IO;
  const uint64_t n = L.values / d;  // a trailing partial point is dropped, as the CSV reader does
  *n_points = n;
  if (!out) return KNNSJ_OK;
  const uint64_t total = n * d;
  // parallel read in 8 MB blocks: each thread opens the file and reads its blocks
  const uint64_t block = (8u << 20) / (uint64_t)L.elem;
  const int64_t nblocks = (int64_t)((total + block - 1) / block);
  int failed = 0;
#pragma omp parallel reduction(| : failed)
  {
    FILE* g = std::fopen(path, "rb");
    if (!g) failed = 1;
    std::vector<unsigned char> buf;
#pragma omp for schedule(dynamic, 4)
    for (int64_t b = 0; b < nblocks; b++) {
      if (!g) continue;
      const uint64_t v0 = (uint64_t)b * block;
      const uint64_t cnt = std::min<uint64_t>(block, total - v0);
      if (std::fseek(g, (long)(L.offset + v0 * (uint64_t)L.elem), SEEK_SET) != 0) {
        failed = 1;
        continue;
      }
      if (L.elem == (int)sizeof(T)) {
        if (std::fread(out + v0, sizeof(T), cnt, g) != cnt) failed = 1;
      } else {
        buf.resize(cnt * (uint64_t)L.elem);
        if (std::fread(buf.data(), 1, buf.size(), g) != buf.size()) {
          failed = 1;
          continue;
        }
        for (uint64_t i = 0; i < cnt; i++) {
          if (L.elem == 4) {
            float v;
            std::memcpy(&v, &buf[i * 4], 4);
            out[v0 + i] = (T)v;
          } else {
            double v;
            std::memcpy(&v, &buf[i * 8], 8);
            out[v0 + i] = (T)v;  // float64 -> float32: round to nearest
          }
        }
      }
    }
    if (g) std::fclose(g);
  }
  return failed ? KNNSJ_ERR_IO : KNNSJ_OK;
}

}  // namespace

extern "C" {

knnsj_status knnsj_read_binary(const char* path, knnsj_dtype dtype, uint32_t d, void* out, uint64_t* n_points) {
  if (!path || !n_points || d == 0) return KNNSJ_ERR_INVALID_ARGUMENT;
  if (dtype == KNNSJ_F32) return read_binary_impl<float>(path, d, (float*)out, n_points);
  if (dtype == KNNSJ_F64) return read_binary_impl<double>(path, d, (double*)out, n_points);
  return KNNSJ_ERR_INVALID_ARGUMENT;
}

knnsj_status knnsj_reorder_dims(const void* data, knnsj_dtype dtype, uint64_t n, uint32_t d, uint32_t* perm,
                                void* variances) {
  if (!data || !perm || n == 0 || d == 0) return KNNSJ_ERR_INVALID_ARGUMENT;
  const uint64_t ns = (n + 99) / 100;
  if (dtype == KNNSJ_F32) {
    std::vector<float> s(ns * d);
    for (uint64_t i = 0; i < ns; i++) std::memcpy(&s[i * d], (const float*)data + i * 100 * d, d * 4);
    reorder_from_sample<float>(s.data(), ns, n, d, perm, (float*)variances);
  } else if (dtype == KNNSJ_F64) {
    std::vector<double> s(ns * d);
    for (uint64_t i = 0; i < ns; i++) std::memcpy(&s[i * d], (const double*)data + i * 100 * d, d * 8);
    reorder_from_sample<double>(s.data(), ns, n, d, perm, (double*)variances);
  } else {
    return KNNSJ_ERR_INVALID_ARGUMENT;
  }
  return KNNSJ_OK;
}

knnsj_status knnsj_grid_dims(const void* data, knnsj_dtype dtype, uint64_t n, uint32_t d, uint32_t di,
                             double eps, void* minArr, void* maxArr, uint32_t* nCells, uint64_t* totalCells) {
  if (!data || !minArr || !maxArr || !nCells || !totalCells || n == 0 || di == 0 || di > d || !(eps > 0))
    return KNNSJ_ERR_INVALID_ARGUMENT;
  if (dtype == KNNSJ_F32)
    grid_dims_host<float>((const float*)data, n, d, di, (float)eps, (float*)minArr, (float*)maxArr, nCells,
                          totalCells);
  else if (dtype == KNNSJ_F64)
    grid_dims_host<double>((const double*)data, n, d, di, eps, (double*)minArr, (double*)maxArr, nCells,
                           totalCells);
  else
    return KNNSJ_ERR_INVALID_ARGUMENT;
  return KNNSJ_OK;
}

knnsj_status knnsj_read_csv(const char* path, knnsj_dtype dtype, uint32_t d, void* out, uint64_t* n_points) {
  if (!path || !n_points || d == 0) return KNNSJ_ERR_INVALID_ARGUMENT;
  if (dtype == KNNSJ_F32) return read_csv_impl<float>(path, d, (float*)out, n_points);
  if (dtype == KNNSJ_F64) return read_csv_impl<double>(path, d, (double*)out, n_points);
  return KNNSJ_ERR_INVALID_ARGUMENT;
}

knnsj_status knnsj_write_knn_out(const char* dir, uint64_t n, uint32_t K, const int32_t* ids, const void* dists,
                                 knnsj_dtype dtype) {
  if (!ids || !dists || K == 0) return KNNSJ_ERR_INVALID_ARGUMENT;
  if (dtype == KNNSJ_F32) return write_knn_out_impl<float>(dir, n, K, ids, (const float*)dists);
  if (dtype == KNNSJ_F64) return write_knn_out_impl<double>(dir, n, K, ids, (const double*)dists);
  return KNNSJ_ERR_INVALID_ARGUMENT;
}

knnsj_status knnsj_write_outlier_scores(const char* dir, uint64_t n, uint32_t K, const int32_t* ids,
                                        const void* dists, knnsj_dtype dtype) {
  if (!ids || !dists || K < 2) return KNNSJ_ERR_INVALID_ARGUMENT;
  if (dtype == KNNSJ_F32) return write_outlier_impl<float>(dir, n, K, ids, (const float*)dists);
  if (dtype == KNNSJ_F64) return write_outlier_impl<double>(dir, n, K, ids, (const double*)dists);
  return KNNSJ_ERR_INVALID_ARGUMENT;
}

}  // extern "C"
