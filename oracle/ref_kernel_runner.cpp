// ref_kernel_runner.cpp -- runs the reference's own range-search kernel.
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
  unsigned int nf = 0;
  RK(cuModuleGetFunctionCount(&nf, mod));
  std::vector<CUfunction> fs(nf);
  RK(cuModuleEnumerateFunctions(fs.data(), nf, mod));
  CUfunction kern = nullptr;
  for (CUfunction f : fs) {
    const char* name = nullptr;
    RK(cuFuncGetName(&name, f));
    if (name && std::strstr(name, "kernelNDGridIndexGlobalkNN")) kern = f;
  }
  if (!kern) {
    std::snprintf(c.err, c.errlen, "kernelNDGridIndexGlobalkNN not in %s", cubin);
    return false;
  }
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

}  // namespace

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
