// ref_kernel_runner.cpp -- runs the reference's own range-search and
// epsilon-estimator kernels.
//
// TEST INFRASTRUCTURE ONLY.  Loads a cubin made by build_ref_kernel.sh from
// the reference's kernel.cu (kernelNDGridIndexGlobalkNN, kernel.cu:61-113,
// with evaluateCell kernel.cu:180-225 and evalPoint kernel.cu:116-161) and
// launches it once over a list of query points with the grid index laid out
// as the reference lays it out (structs.h:119-133): grid{indexmin,indexmax}
// per non-empty cell, gridCellLookup{idx, gridLinearID} sorted by linear id,
// the point lookup array, minArr and nCells -- the arrays the CPU oracle's
// grid builder produces and tests pin against the reference's host code.
// The kernel appends every (query, point, distance) within epsilon to three
// arrays through an atomic counter (kernel.cu:149-153); they are returned
// unsorted.  Only tests use this, to pin the oracle's distance arithmetic,
// within-radius rule and ring coverage against the reference kernel run on
// the GPU.  It uses the CUDA driver API so that the kernel needs no host
// code of the reference.
#include <cuda.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

struct GridCell {  // struct grid, structs.h:119-122
  int indexmin;
  int indexmax;
};
struct GridCellLookup {  // struct gridCellLookup, structs.h:126-133
  unsigned int idx;
  uint64_t gridLinearID;
};

struct Ctx {
  char* err;
  int errlen;
  bool fail(const char* what, CUresult r) {
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    std::snprintf(err, errlen, "%s: %s", what, s ? s : "?");
    return false;
  }
};

#define RK(call)                                      \
  do {                                                \
    CUresult r_ = (call);                             \
    if (r_ != CUDA_SUCCESS) return c.fail(#call, r_); \
  } while (0)

struct DevMem {
  CUdeviceptr p = 0;
  ~DevMem() {
    if (p) cuMemFree(p);
  }
};

CUfunction find_kernel(Ctx& c, CUmodule mod, const char* want);

bool upload(Ctx& c, DevMem& m, const void* src, size_t bytes) {
  RK(cuMemAlloc(&m.p, bytes < 16 ? 16 : bytes));
  if (src && bytes) RK(cuMemcpyHtoD(m.p, src, bytes));
  return true;
}

bool run(Ctx& c, const char* cubin, int tbytes, const void* data, uint64_t n, uint32_t d, const void* eps,
         const void* minArr, const uint32_t* nCells, uint32_t di, const uint64_t* cellKeys, const int32_t* imin,
         const int32_t* imax, uint64_t nne, const uint32_t* lookup, const uint32_t* queries, uint32_t nq,
         uint32_t tpp, uint64_t cap, int32_t* out_q, int32_t* out_p, void* out_dist, uint64_t* out_count) {
  RK(cuInit(0));
  CUdevice dev;
  RK(cuDeviceGet(&dev, 0));
  CUcontext ctx;
  RK(cuDevicePrimaryCtxRetain(&ctx, dev));
  RK(cuCtxSetCurrent(ctx));
  CUmodule mod;
  RK(cuModuleLoad(&mod, cubin));
  CUfunction kern = find_kernel(c, mod, "kernelNDGridIndexGlobalkNN");
  if (!kern) return false;
  std::vector<GridCell> grid(nne);
  std::vector<GridCellLookup> gcl(nne);
  for (uint64_t i = 0; i < nne; i++) {
    grid[i].indexmin = imin[i];
    grid[i].indexmax = imax[i];
    gcl[i].idx = (unsigned int)i;
    gcl[i].gridLinearID = cellKeys[i];
  }
  const unsigned int zero = 0, one = 1, kk = 0, N = nq, nne32 = (unsigned int)nne, tpp32 = tpp;
  const unsigned long long work[2] = {0, 0};
  DevMem dbg1, dbg2, dk, dN, doff, dbatch, ddata, deps, dindex, dlookup, dgcl, dmin, dncells, dcnt, dnne, dpik, dpiv,
      ddist, dq, dtpp, dwork;
  bool ok = upload(c, dbg1, &zero, 4) && upload(c, dbg2, &zero, 4) && upload(c, dk, &kk, 4) &&
            upload(c, dN, &N, 4) && upload(c, doff, &one, 4) && upload(c, dbatch, &zero, 4) &&
            upload(c, ddata, data, n * d * tbytes) && upload(c, deps, eps, tbytes) &&
            upload(c, dindex, grid.data(), nne * sizeof(GridCell)) && upload(c, dlookup, lookup, n * 4) &&
            upload(c, dgcl, gcl.data(), nne * sizeof(GridCellLookup)) && upload(c, dmin, minArr, di * tbytes) &&
            upload(c, dncells, nCells, di * 4) && upload(c, dcnt, &zero, 4) && upload(c, dnne, &nne32, 4) &&
            upload(c, dpik, nullptr, cap * 4) && upload(c, dpiv, nullptr, cap * 4) &&
            upload(c, ddist, nullptr, cap * tbytes) && upload(c, dq, queries, (size_t)nq * 4) &&
            upload(c, dtpp, &tpp32, 4) && upload(c, dwork, work, sizeof(work));
  if (!ok) return false;
  void* args[] = {&dbg1.p, &dbg2.p, &dk.p,    &dN.p,  &doff.p, &dbatch.p, &ddata.p,
                  &deps.p, &dindex.p, &dlookup.p, &dgcl.p, &dmin.p, &dncells.p, &dcnt.p,
                  &dnne.p, &dpik.p, &dpiv.p, &ddist.p, &dq.p, &dtpp.p, &dwork.p};
  const unsigned int block = 256;  // BLOCKSIZE, params.h:72
  const uint64_t threads = (uint64_t)nq * tpp;
  const unsigned int blocks = (unsigned int)((threads + block - 1) / block);
  RK(cuLaunchKernel(kern, blocks, 1, 1, block, 1, 1, 0, nullptr, args, nullptr));
  RK(cuCtxSynchronize());
  unsigned int cnt = 0;
  RK(cuMemcpyDtoH(&cnt, dcnt.p, 4));
  *out_count = cnt;
  if (cnt > cap) {
    std::snprintf(c.err, c.errlen, "pair count %u above capacity %llu", cnt, (unsigned long long)cap);
    return false;
  }
  RK(cuMemcpyDtoH(out_q, dpik.p, (size_t)cnt * 4));
  RK(cuMemcpyDtoH(out_p, dpiv.p, (size_t)cnt * 4));
  RK(cuMemcpyDtoH(out_dist, ddist.p, (size_t)cnt * tbytes));
  RK(cuModuleUnload(mod));
  return true;
}

CUfunction find_kernel(Ctx& c, CUmodule mod, const char* want) {
  unsigned int nf = 0;
  if (cuModuleGetFunctionCount(&nf, mod) != CUDA_SUCCESS) return nullptr;
  std::vector<CUfunction> fs(nf);
  if (cuModuleEnumerateFunctions(fs.data(), nf, mod) != CUDA_SUCCESS) return nullptr;
  for (CUfunction f : fs) {
    const char* name = nullptr;
    if (cuFuncGetName(&name, f) == CUDA_SUCCESS && name && std::strstr(name, want)) return f;
  }
  std::snprintf(c.err, c.errlen, "%s not in the cubin", want);
  return nullptr;
}

// The epsilon estimator's two kernels (kernel.cu:343-381, 450-523) with the
// reference's launch shapes (GPU.cu:3275-3290, 3440-3456): the sampled mean
// distance (an unordered double atomic sum, so only its count is exact) and
// the 10 000-bucket histogram, the latter run with the caller's mean and
// bucket width so that its integer counts can be compared exactly.
bool run_eps(Ctx& c, const char* cubin, int tbytes, const void* data, uint64_t n, uint32_t d, double avg_in,
             double bucket_width, uint32_t offset, uint32_t* hist_out, double* total_out,
             unsigned long long* cnt_out) {
  RK(cuInit(0));
  CUdevice dev;
  RK(cuDeviceGet(&dev, 0));
  CUcontext ctx;
  RK(cuDevicePrimaryCtxRetain(&ctx, dev));
  RK(cuCtxSetCurrent(ctx));
  CUmodule mod;
  RK(cuModuleLoad(&mod, cubin));
  CUfunction kavg = find_kernel(c, mod, "kernelEstimateAvgDistBruteForce");
  CUfunction khist = find_kernel(c, mod, "kernelKDistBruteForce");
  if (!kavg || !khist) return false;
  const unsigned int N = (unsigned int)n, zero = 0, off = offset;
  const unsigned long long zero64 = 0;
  const double dz = 0.0;
  // one spare bucket: a distance just below the mean can round to bucket
  // 10000, which the reference writes without a check (kernel.cu:511-512)
  std::vector<uint32_t> hz(10001, 0);
  DevMem dN, dbg1, dbg2, dcnt, ddata, dtot, doff, dcnt2, davg, dhist, dbw;
  bool ok = upload(c, dN, &N, 4) && upload(c, dbg1, &zero, 4) && upload(c, dbg2, &zero, 4) &&
            upload(c, dcnt, &zero64, 8) && upload(c, ddata, data, n * d * tbytes) && upload(c, dtot, &dz, 8) &&
            upload(c, doff, &off, 4) && upload(c, dcnt2, &zero64, 8) && upload(c, davg, &avg_in, 8) &&
            upload(c, dhist, hz.data(), hz.size() * 4) && upload(c, dbw, &bucket_width, 8);
  if (!ok) return false;
  const unsigned int block = 256;
  // GPU.cu:3275: TOTALBLOCKS = ceil((0.001*N)/(1.0*BLOCKSIZE))
  const unsigned int blocks_avg = (unsigned int)std::ceil((0.001 * N) / (1.0 * block));
  void* a_avg[] = {&dN.p, &dbg1.p, &dbg2.p, &dcnt.p, &ddata.p, &dtot.p};
  RK(cuLaunchKernel(kavg, blocks_avg, 1, 1, block, 1, 1, 0, nullptr, a_avg, nullptr));
  const unsigned int blocks_hist = N / offset;  // GPU.cu:3434: ceil((*N)/(*offset)) of an integer quotient
  void* a_hist[] = {&dN.p, &doff.p, &dbg1.p, &dbg2.p, &dcnt2.p, &ddata.p, &davg.p, &dhist.p, &dbw.p};
  if (blocks_hist > 0) RK(cuLaunchKernel(khist, blocks_hist, 1, 1, block, 1, 1, 0, nullptr, a_hist, nullptr));
  RK(cuCtxSynchronize());
  RK(cuMemcpyDtoH(total_out, dtot.p, 8));
  RK(cuMemcpyDtoH(cnt_out, dcnt.p, 8));
  RK(cuMemcpyDtoH(hist_out, dhist.p, 10001 * 4));
  RK(cuModuleUnload(mod));
  return true;
}

}  // namespace

extern "C" int refk_eps(const char* cubin, int tbytes, const void* data, uint64_t n, uint32_t d, double avg_in,
                        double bucket_width, uint32_t offset, uint32_t* hist_out /*10001*/, double* total_out,
                        unsigned long long* cnt_out, char* err, int errlen) {
  Ctx c{err, errlen};
  if (err && errlen > 0) err[0] = 0;
  if (n % 256 != 0 || offset == 0) {
    // the histogram kernel reads up to 255 points past the last stride
    // (kernel.cu:486-492); a multiple of 256 points keeps every read in range
    std::snprintf(err, errlen, "n must be a multiple of 256 and offset positive");
    return 1;
  }
  return run_eps(c, cubin, tbytes, data, n, d, avg_in, bucket_width, offset, hist_out, total_out, cnt_out) ? 0 : 1;
}

extern "C" int refk_run(const char* cubin, int tbytes, const void* data, uint64_t n, uint32_t d, const void* eps,
                        const void* minArr, const uint32_t* nCells, uint32_t di, const uint64_t* cellKeys,
                        const int32_t* imin, const int32_t* imax, uint64_t nne, const uint32_t* lookup,
                        const uint32_t* queries, uint32_t nq, uint32_t threads_per_point, uint64_t capacity,
                        int32_t* out_q, int32_t* out_p, void* out_dist, uint64_t* out_count, char* err,
                        int errlen) {
  Ctx c{err, errlen};
  if (err && errlen > 0) err[0] = 0;
  if (capacity >= (1ull << 32)) {
    std::snprintf(err, errlen, "capacity above 2^32-1 (the kernel's counter is 32-bit)");
    return 1;
  }
  return run(c, cubin, tbytes, data, n, d, eps, minArr, nCells, di, cellKeys, imin, imax, nne, lookup, queries,
             nq, threads_per_point, capacity, out_q, out_p, out_dist, out_count)
             ? 0
             : 1;
}
