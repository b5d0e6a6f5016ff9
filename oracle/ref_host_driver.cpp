// ref_host_driver.cpp -- drives the reference's own HOST functions, compiled
// from the reference sources by oracle/build_ref_host.sh, to produce golden
// fixtures for the oracle and the product's host pipeline.
//
// TEST INFRASTRUCTURE ONLY: linked with objects built from the reference's
// main.cu / GPU.cu / kernel.cu / import_dataset.cpp / par_sort.cpp into
// oracle/_ref/.  Only host functions that touch no GPU are called:
//   ReorderByDimension                         (main.cu:2521)
//   generateNDGridDimensions                   (main.cu:2425)
//   populateNDGridIndexAndLookupArrayParallel  (main.cu:1968)
//   computeWorkDifficulty                      (main.cu:2941)
//   importNDDataset                            (import_dataset.cpp:50)
//   printNeighborTable                         (main.cu:911)
//   printOutlierScores                         (main.cu:952)
//
// The two index types below repeat the layout of the reference's `grid` and
// `gridCellLookup` (structs.h:119-133) so the calls link and read the same
// memory; DTYPE comes from the build (-DREF_DTYPE=float|double).
//
// Usage:
//   ref_host_driver prep  <in.bin> <eps> <out_prefix>
//   ref_host_driver csv   <file.csv> <out.bin>
//   ref_host_driver print <table.bin> <out_dir>
// Binary arrays are raw little-endian; <in.bin> holds uint64 n, uint32 d,
// then n*d DTYPE values row-major.

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <unistd.h>
#include <vector>

#ifndef REF_DTYPE
#define REF_DTYPE float
#endif
typedef REF_DTYPE dtype_t;

struct grid {
  int indexmin;
  int indexmax;
};
struct gridCellLookup {
  unsigned int idx;
  uint64_t gridLinearID;
};

void ReorderByDimension(std::vector<std::vector<dtype_t> >* NDdataPoints);
void generateNDGridDimensions(std::vector<std::vector<dtype_t> >* NDdataPoints, dtype_t epsilon,
                              dtype_t* minArr, dtype_t* maxArr, unsigned int* nCells,
                              uint64_t* totalCells);
void populateNDGridIndexAndLookupArrayParallel(std::vector<std::vector<dtype_t> >* NDdataPoints,
                                               dtype_t epsilon, struct gridCellLookup** gridCellLookupArr,
                                               struct grid** index, unsigned int* indexLookupArr,
                                               dtype_t* minArr, unsigned int* nCells,
                                               uint64_t totalCells, unsigned int* nNonEmptyCells);
void computeWorkDifficulty(unsigned int* outputOrderedQueryPntIDs, struct gridCellLookup* gridCellLookupArr,
                           unsigned int* nNonEmptyCells, unsigned int* indexLookupArr, struct grid* index);
void importNDDataset(std::vector<std::vector<dtype_t> >* dataPoints, char* fname);
void printNeighborTable(unsigned int databaseSize, int k_Neighbors, int* nearestNeighborTable,
                        dtype_t* nearestNeighborTableDistances);
void printOutlierScores(unsigned int databaseSize, int k_Neighbors, int* nearestNeighborTable,
                        dtype_t* nearestNeighborTableDistances);

static void die(const char* m) {
  fprintf(stderr, "ref_host_driver: %s\n", m);
  exit(2);
}

template <typename X>
static void write_arr(const std::string& path, const X* p, size_t n) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) die("cannot write output");
  if (n && fwrite(p, sizeof(X), n, f) != n) die("short write");
  fclose(f);
}

static std::vector<std::vector<dtype_t> > read_points(const char* path, uint32_t* d_out) {
  FILE* f = fopen(path, "rb");
  if (!f) die("cannot open input");
  uint64_t n;
  uint32_t d;
  if (fread(&n, 8, 1, f) != 1 || fread(&d, 4, 1, f) != 1) die("bad header");
  std::vector<dtype_t> flat(n * d);
  if (fread(flat.data(), sizeof(dtype_t), flat.size(), f) != flat.size()) die("short read");
  fclose(f);
  std::vector<std::vector<dtype_t> > pts(n);
  for (uint64_t i = 0; i < n; i++) pts[i].assign(flat.begin() + i * d, flat.begin() + (i + 1) * d);
  *d_out = d;
  return pts;
}

int main(int argc, char** argv) {
  if (argc < 2) die("missing command");
  std::string cmd = argv[1];
  // the reference's functions print progress on stdout; keep it off ours
  if (!freopen("/dev/null", "w", stdout)) die("freopen");
  if (cmd == "prep") {
    if (argc != 5) die("prep <in.bin> <eps> <out_prefix>");
    uint32_t d;
    std::vector<std::vector<dtype_t> > pts = read_points(argv[2], &d);
    const dtype_t eps = (dtype_t)atof(argv[3]);
    const std::string out = argv[4];
    const size_t n = pts.size();
    ReorderByDimension(&pts);
    std::vector<dtype_t> flat;
    flat.reserve(n * d);
    for (auto& p : pts) flat.insert(flat.end(), p.begin(), p.end());
    write_arr(out + "reordered.bin", flat.data(), flat.size());
    const int di = NUMINDEXEDDIM_BUILD;
    std::vector<dtype_t> minArr(di), maxArr(di);
    std::vector<unsigned int> nCells(di);
    uint64_t totalCells = 0;
    generateNDGridDimensions(&pts, eps, minArr.data(), maxArr.data(), nCells.data(), &totalCells);
    write_arr(out + "minArr.bin", minArr.data(), di);
    write_arr(out + "maxArr.bin", maxArr.data(), di);
    write_arr(out + "nCells.bin", nCells.data(), di);
    write_arr(out + "totalCells.bin", &totalCells, 1);
    struct gridCellLookup* lookupArr = nullptr;
    struct grid* index = nullptr;
    std::vector<unsigned int> indexLookupArr(n);
    unsigned int nNonEmpty = 0;
    populateNDGridIndexAndLookupArrayParallel(&pts, eps, &lookupArr, &index, indexLookupArr.data(),
                                              minArr.data(), nCells.data(), totalCells, &nNonEmpty);
    std::vector<uint64_t> keys(nNonEmpty);
    std::vector<uint32_t> idx(nNonEmpty);
    std::vector<int32_t> imin(nNonEmpty), imax(nNonEmpty);
    for (unsigned int c = 0; c < nNonEmpty; c++) {
      keys[c] = lookupArr[c].gridLinearID;
      idx[c] = lookupArr[c].idx;
      imin[c] = index[c].indexmin;
      imax[c] = index[c].indexmax;
    }
    write_arr(out + "cellKeys.bin", keys.data(), keys.size());
    write_arr(out + "cellIdx.bin", idx.data(), idx.size());
    write_arr(out + "indexmin.bin", imin.data(), imin.size());
    write_arr(out + "indexmax.bin", imax.data(), imax.size());
    write_arr(out + "lookup.bin", indexLookupArr.data(), n);
    std::vector<unsigned int> order(n);
    computeWorkDifficulty(order.data(), lookupArr, &nNonEmpty, indexLookupArr.data(), index);
    write_arr(out + "workorder.bin", order.data(), n);
    return 0;
  }
  if (cmd == "csv") {
    if (argc != 4) die("csv <file.csv> <out.bin>");
    std::vector<std::vector<dtype_t> > pts;
    importNDDataset(&pts, argv[2]);
    std::vector<dtype_t> flat;
    for (auto& p : pts) flat.insert(flat.end(), p.begin(), p.end());
    uint64_t n = pts.size();
    FILE* f = fopen(argv[3], "wb");
    if (!f) die("cannot write");
    fwrite(&n, 8, 1, f);
    if (!flat.empty()) fwrite(flat.data(), sizeof(dtype_t), flat.size(), f);
    fclose(f);
    return 0;
  }
  if (cmd == "print") {
    // <table.bin>: uint64 n, uint32 K, then n*K int32 ids, n*K DTYPE dists
    if (argc != 4) die("print <table.bin> <out_dir>");
    FILE* f = fopen(argv[2], "rb");
    if (!f) die("cannot open table");
    uint64_t n;
    uint32_t K;
    if (fread(&n, 8, 1, f) != 1 || fread(&K, 4, 1, f) != 1) die("bad header");
    std::vector<int> ids(n * K);
    std::vector<dtype_t> dists(n * K);
    if (fread(ids.data(), 4, ids.size(), f) != ids.size()) die("short ids");
    if (fread(dists.data(), sizeof(dtype_t), dists.size(), f) != dists.size()) die("short dists");
    fclose(f);
    if (chdir(argv[3]) != 0) die("chdir");
    printNeighborTable((unsigned int)n, (int)K, ids.data(), dists.data());
    printOutlierScores((unsigned int)n, (int)K, ids.data(), dists.data());
    return 0;
  }
  die("unknown command");
  return 2;
}
