/*
 * refshim.c -- runs the reference's own kernels on the GPU (TEST INFRASTRUCTURE).
 *
 * oracle/build: the reference's kernels/briefmatch_cuda.cu and kernels/util_cuda.cu
 * are compiled, unmodified and with the reference's nvcc flags (-O3 -use_fast_math),
 * to sm_103a cubins in oracle/_ref/.  The reference host code cannot be built here
 * (it needs OpenCV, Boost and libpng), so this shim replaces its launchers
 * (briefmatch_cuda.cu:300-380, util_cuda.cu:185-282): it loads the cubins with the
 * CUDA driver API and launches each kernel with the reference's 32x32 blocks on
 * the default stream, synchronising after each launch as the reference does.
 * Buffers are allocated by the caller with size_t sizes and guard bands, which
 * replaces the reference's int-sized CUDA_constructor (util_cuda.cu:206-210).
 *
 * Used only by the tests and bench.py's reference leg, as the comparison
 * baseline; the engine never calls it.
 */
#include <cuda.h>
#include <dlfcn.h>
#include <stdio.h>
#include <string.h>

typedef CUresult (*fn_cuInit)(unsigned int);
typedef CUresult (*fn_cuDeviceGet)(CUdevice*, int);
typedef CUresult (*fn_cuDevicePrimaryCtxRetain)(CUcontext*, CUdevice);
typedef CUresult (*fn_cuCtxSetCurrent)(CUcontext);
typedef CUresult (*fn_cuCtxSynchronize)(void);
typedef CUresult (*fn_cuModuleLoad)(CUmodule*, const char*);
typedef CUresult (*fn_cuModuleGetFunctionCount)(unsigned int*, CUmodule);
typedef CUresult (*fn_cuModuleEnumerateFunctions)(CUfunction*, unsigned int, CUmodule);
typedef CUresult (*fn_cuFuncGetName)(const char**, CUfunction);
typedef CUresult (*fn_cuModuleGetGlobal)(CUdeviceptr*, size_t*, CUmodule, const char*);
typedef CUresult (*fn_cuMemcpyHtoD)(CUdeviceptr, const void*, size_t);
typedef CUresult (*fn_cuLaunchKernel)(CUfunction, unsigned int, unsigned int, unsigned int, unsigned int,
                                      unsigned int, unsigned int, unsigned int, CUstream, void**, void**);
typedef CUresult (*fn_cuGetErrorString)(CUresult, const char**);

static struct {
    void* h;
    fn_cuInit Init;
    fn_cuDeviceGet DeviceGet;
    fn_cuDevicePrimaryCtxRetain PrimaryCtxRetain;
    fn_cuCtxSetCurrent CtxSetCurrent;
    fn_cuCtxSynchronize CtxSynchronize;
    fn_cuModuleLoad ModuleLoad;
    fn_cuModuleGetFunctionCount GetFunctionCount;
    fn_cuModuleEnumerateFunctions EnumerateFunctions;
    fn_cuFuncGetName FuncGetName;
    fn_cuModuleGetGlobal GetGlobal;
    fn_cuMemcpyHtoD MemcpyHtoD;
    fn_cuLaunchKernel LaunchKernel;
    fn_cuGetErrorString GetErrorString;
    CUmodule mod_bm, mod_util;
    CUfunction f_initRandom, f_binaryFeatures, f_init, f_propagate, f_randomSearch, f_cbFilter;
    CUfunction f_filterConst, f_medianFilter1D, f_mult, f_resizeLanczos, f_resizeNN, f_convert;
    int loaded;
} g;

static char g_err[512];

const char* rs_error(void) { return g_err; }

static int cu_fail(CUresult r, const char* what)
{
    const char* s = "unknown";
    if (g.GetErrorString) g.GetErrorString(r, &s);
    snprintf(g_err, sizeof(g_err), "%s: %s (%d)", what, s, (int)r);
    return -1;
}

#define CU(call, what)                      \
    do {                                    \
        CUresult r_ = (call);               \
        if (r_ != CUDA_SUCCESS) return cu_fail(r_, what); \
    } while (0)

static void* sym(const char* a, const char* b)
{
    void* p = dlsym(g.h, a);
    if (!p && b) p = dlsym(g.h, b);
    return p;
}

/* Kernel whose mangled name holds "<len><name>" with no digit before the length. */
static CUfunction find_kernel(CUmodule m, const char* name)
{
    char key[64];
    snprintf(key, sizeof(key), "%d%s", (int)strlen(name), name);
    unsigned int n = 0;
    if (g.GetFunctionCount(&n, m) != CUDA_SUCCESS || n == 0 || n > 256) return NULL;
    CUfunction fs[256];
    if (g.EnumerateFunctions(fs, n, m) != CUDA_SUCCESS) return NULL;
    for (unsigned int i = 0; i < n; i++) {
        const char* fname = NULL;
        if (g.FuncGetName(&fname, fs[i]) != CUDA_SUCCESS || !fname) continue;
        const char* hit = strstr(fname, key);
        while (hit) {
            if (hit == fname || !(hit[-1] >= '0' && hit[-1] <= '9')) return fs[i];
            hit = strstr(hit + 1, key);
        }
    }
    return NULL;
}

int rs_load(const char* bm_cubin, const char* util_cubin)
{
    if (g.loaded) return 0;
    g.h = dlopen("libcuda.so.1", RTLD_NOW | RTLD_GLOBAL);
    if (!g.h) {
        snprintf(g_err, sizeof(g_err), "dlopen libcuda.so.1 failed");
        return -1;
    }
    g.Init = (fn_cuInit)sym("cuInit", NULL);
    g.DeviceGet = (fn_cuDeviceGet)sym("cuDeviceGet", NULL);
    g.PrimaryCtxRetain = (fn_cuDevicePrimaryCtxRetain)sym("cuDevicePrimaryCtxRetain", NULL);
    g.CtxSetCurrent = (fn_cuCtxSetCurrent)sym("cuCtxSetCurrent", NULL);
    g.CtxSynchronize = (fn_cuCtxSynchronize)sym("cuCtxSynchronize", NULL);
    g.ModuleLoad = (fn_cuModuleLoad)sym("cuModuleLoad", NULL);
    g.GetFunctionCount = (fn_cuModuleGetFunctionCount)sym("cuModuleGetFunctionCount", NULL);
    g.EnumerateFunctions = (fn_cuModuleEnumerateFunctions)sym("cuModuleEnumerateFunctions", NULL);
    g.FuncGetName = (fn_cuFuncGetName)sym("cuFuncGetName", NULL);
    g.GetGlobal = (fn_cuModuleGetGlobal)sym("cuModuleGetGlobal_v2", "cuModuleGetGlobal");
    g.MemcpyHtoD = (fn_cuMemcpyHtoD)sym("cuMemcpyHtoD_v2", "cuMemcpyHtoD");
    g.LaunchKernel = (fn_cuLaunchKernel)sym("cuLaunchKernel", NULL);
    g.GetErrorString = (fn_cuGetErrorString)sym("cuGetErrorString", NULL);
    if (!g.Init || !g.DeviceGet || !g.PrimaryCtxRetain || !g.CtxSetCurrent || !g.CtxSynchronize || !g.ModuleLoad ||
        !g.GetFunctionCount || !g.EnumerateFunctions || !g.FuncGetName || !g.GetGlobal || !g.MemcpyHtoD ||
        !g.LaunchKernel) {
        snprintf(g_err, sizeof(g_err), "driver entry point missing");
        return -1;
    }
    CU(g.Init(0), "cuInit");
    CUdevice dev;
    CU(g.DeviceGet(&dev, 0), "cuDeviceGet");
    CUcontext ctx;
    CU(g.PrimaryCtxRetain(&ctx, dev), "cuDevicePrimaryCtxRetain");
    CU(g.CtxSetCurrent(ctx), "cuCtxSetCurrent");
    CU(g.ModuleLoad(&g.mod_bm, bm_cubin), "cuModuleLoad(briefmatch_cuda)");
    CU(g.ModuleLoad(&g.mod_util, util_cubin), "cuModuleLoad(util_cuda)");
    struct { CUfunction* f; CUmodule* m; const char* n; } ks[] = {
        {&g.f_initRandom, &g.mod_bm, "initRandom"},    {&g.f_binaryFeatures, &g.mod_bm, "binaryFeatures"},
        {&g.f_init, &g.mod_bm, "init"},                {&g.f_propagate, &g.mod_bm, "propagate"},
        {&g.f_randomSearch, &g.mod_bm, "randomSearch"}, {&g.f_cbFilter, &g.mod_bm, "cbFilter"},
        {&g.f_filterConst, &g.mod_util, "filterConst"}, {&g.f_medianFilter1D, &g.mod_util, "medianFilter1D"},
        {&g.f_mult, &g.mod_util, "mult"},              {&g.f_resizeLanczos, &g.mod_util, "resizeLanczos"},
        {&g.f_resizeNN, &g.mod_util, "resizeNN"},      {&g.f_convert, &g.mod_util, "convert"},
    };
    for (size_t i = 0; i < sizeof(ks) / sizeof(ks[0]); i++) {
        *ks[i].f = find_kernel(*ks[i].m, ks[i].n);
        if (!*ks[i].f) {
            snprintf(g_err, sizeof(g_err), "reference kernel %s not found in its cubin", ks[i].n);
            return -1;
        }
    }
    g.loaded = 1;
    return 0;
}

static int launch(CUfunction f, int sx, int sy, void** args, const char* what)
{
    if (!g.loaded) {
        snprintf(g_err, sizeof(g_err), "refshim not loaded");
        return -1;
    }
    unsigned int bx = (unsigned)((sx + 31) / 32), by = (unsigned)((sy + 31) / 32);
    CU(g.LaunchKernel(f, bx, by, 1, 32, 32, 1, 0, NULL, args, NULL), what);
    CU(g.CtxSynchronize(), what);
    return 0;
}

/* CUDA_copyPatchToConst, briefmatch_cuda.cu:376-379 (2048 floats). */
int rs_set_pattern(const float* pattern2048)
{
    CUdeviceptr p;
    size_t bytes;
    CU(g.GetGlobal(&p, &bytes, g.mod_bm, "const_sampPatch"), "const_sampPatch");
    if (bytes < 2048 * sizeof(float)) return cu_fail(CUDA_ERROR_INVALID_VALUE, "const_sampPatch size");
    CU(g.MemcpyHtoD(p, pattern2048, 2048 * sizeof(float)), "copy pattern");
    return 0;
}

/* CUDA_copyToConst, util_cuda.cu:277-280 (100 floats). */
int rs_set_kernel(const float* kernel100)
{
    CUdeviceptr p;
    size_t bytes;
    CU(g.GetGlobal(&p, &bytes, g.mod_util, "const_kernel"), "const_kernel");
    if (bytes < 100 * sizeof(float)) return cu_fail(CUDA_ERROR_INVALID_VALUE, "const_kernel size");
    CU(g.MemcpyHtoD(p, kernel100, 100 * sizeof(float)), "copy taps");
    return 0;
}

int rs_init_random(CUdeviceptr state, int sx, int sy)
{
    unsigned int usx = (unsigned)sx, usy = (unsigned)sy;
    void* a[] = {&state, &usx, &usy};
    return launch(g.f_initRandom, sx, sy, a, "initRandom");
}

int rs_binary_features(CUdeviceptr I, CUdeviceptr F, int sx, int sy, int N, int Ns)
{
    void* a[] = {&I, &F, &sx, &sy, &N, &Ns};
    return launch(g.f_binaryFeatures, sx, sy, a, "binaryFeatures");
}

int rs_initialize(CUdeviceptr I1, CUdeviceptr I2, CUdeviceptr F1, CUdeviceptr F2, CUdeviceptr D, CUdeviceptr NX,
                  CUdeviceptr NY, int sx, int sy, int first, int N, int Ns)
{
    unsigned char b = first ? 1 : 0;
    void* a[] = {&I1, &I2, &F1, &F2, &D, &NX, &NY, &sx, &sy, &b, &N, &Ns};
    return launch(g.f_init, sx, sy, a, "init");
}

int rs_propagate(CUdeviceptr I1, CUdeviceptr I2, CUdeviceptr F1, CUdeviceptr F2, CUdeviceptr D, CUdeviceptr NX,
                 CUdeviceptr NY, int sx, int sy, int pd, int jfMax, int doubleProp, int N, int Ns)
{
    unsigned char b = doubleProp ? 1 : 0;
    void* a[] = {&I1, &I2, &F1, &F2, &D, &NX, &NY, &sx, &sy, &pd, &jfMax, &b, &N, &Ns};
    return launch(g.f_propagate, sx, sy, a, "propagate");
}

int rs_random_search(CUdeviceptr I1, CUdeviceptr I2, CUdeviceptr F1, CUdeviceptr F2, CUdeviceptr D, CUdeviceptr NX,
                     CUdeviceptr NY, CUdeviceptr state, int sx, int sy, float dist, int N, int Ns)
{
    void* a[] = {&I1, &I2, &F1, &F2, &D, &NX, &NY, &state, &sx, &sy, &dist, &N, &Ns};
    return launch(g.f_randomSearch, sx, sy, a, "randomSearch");
}

int rs_cb_filter(CUdeviceptr Ui, CUdeviceptr Vi, CUdeviceptr Uo, CUdeviceptr Vo, CUdeviceptr Uim, CUdeviceptr Vim,
                 CUdeviceptr I, float sE, float sI, float sS, int sx, int sy)
{
    void* a[] = {&Ui, &Vi, &Uo, &Vo, &Uim, &Vim, &I, &sE, &sI, &sS, &sx, &sy};
    return launch(g.f_cbFilter, sx, sy, a, "cbFilter");
}

int rs_filter_const(CUdeviceptr Li, CUdeviceptr Lo, int ks, int dir, int sx, int sy)
{
    void* a[] = {&Li, &Lo, &ks, &dir, &sx, &sy};
    return launch(g.f_filterConst, sx, sy, a, "filterConst");
}

int rs_median(CUdeviceptr Li, CUdeviceptr Lo, int dir, int fsize, int sx, int sy)
{
    void* a[] = {&Li, &Lo, &dir, &fsize, &sx, &sy};
    return launch(g.f_medianFilter1D, sx, sy, a, "medianFilter1D");
}

int rs_resize_lanczos(CUdeviceptr Li, CUdeviceptr Lo, int sxi, int syi, int sxo, int syo)
{
    void* a[] = {&Li, &Lo, &sxi, &syi, &sxo, &syo};
    return launch(g.f_resizeLanczos, sxo, syo, a, "resizeLanczos");
}

int rs_resize_nn(CUdeviceptr Li, CUdeviceptr Lo, int sxi, int syi, int sxo, int syo)
{
    void* a[] = {&Li, &Lo, &sxi, &syi, &sxo, &syo};
    return launch(g.f_resizeNN, sxo, syo, a, "resizeNN");
}

int rs_mult(CUdeviceptr L, float m, int sx, int sy)
{
    void* a[] = {&L, &m, &sx, &sy};
    return launch(g.f_mult, sx, sy, a, "mult");
}

int rs_convert(CUdeviceptr Li, CUdeviceptr Lo, int sx, int sy)
{
    void* a[] = {&Li, &Lo, &sx, &sy};
    return launch(g.f_convert, sx, sy, a, "convert");
}
