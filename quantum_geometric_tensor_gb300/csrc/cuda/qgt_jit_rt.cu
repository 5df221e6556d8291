// qgt_jit_rt.cu -- compiles the straight-line pass kernels that qgt_jit.c
// writes, loads them and launches them.
//
// Compiler: NVRTC for sm_103a (the same CUDA toolkit as the library).  The
// source handed to it is a short prologue (integer typedefs, the generator
// codes), the gate routines of qgt_pass2_ops.cuh (embedded into the library
// at build time) and the generated kernel.  Compiled images are kept per
// process (keyed by a 64-bit FNV-1a hash of the full source and the compile
// options) and, when a writable cache directory exists ($QGT_JIT_CACHE_DIR,
// else $HOME/.cache/qgt_gb300_jit), on disk, so a plan whose programs were
// compiled before costs no compile time.  Images are loaded with
// cudaLibraryLoadData (context-independent) and stay loaded until exit.
#include <cuda_runtime.h>
#include <errno.h>
#include <nvrtc.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>
#include <unistd.h>

#include "../qgt_internal.h"
#include "qgt_pass2_ops_src.h"   // qgt_pass2_ops_src: the text of qgt_pass2_ops.cuh (generated at build time)

static const char* jit_prologue =
    "typedef unsigned int uint32_t;\n"
    "typedef int int32_t;\n"
    "typedef unsigned long long uint64_t;\n"
    "typedef long long int64_t;\n"
    "typedef signed char int8_t;\n"
    "typedef unsigned char uint8_t;\n"
    "enum { QGEN_NONE = 0, QGEN_X = 1, QGEN_Y = 2, QGEN_Z = 3 };\n";

static const char* jit_opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "-default-device"};
#define JIT_NOPTS 3

struct qgt_jit_kernel {
    uint64_t key;
    cudaLibrary_t lib;
    cudaKernel_t kern;
    int32_t smem;
    int32_t nthreads;        // block size: 32 << warp bits of the tile
    int32_t attr_dev_mask;   // devices (bit per ordinal < 32) whose shared-memory limit is raised
    struct qgt_jit_kernel* next;
};

static pthread_mutex_t jit_mu = PTHREAD_MUTEX_INITIALIZER;
static struct qgt_jit_kernel* jit_list = NULL;
static double jit_seconds = 0.0;

extern "C" double qgt_dev_jit_compile_seconds(void)
{
    pthread_mutex_lock(&jit_mu);
    const double s = jit_seconds;
    pthread_mutex_unlock(&jit_mu);
    return s;
}

static uint64_t fnv1a(uint64_t h, const char* s, size_t n)
{
    for (size_t i = 0; i < n; i++) {
        h ^= (unsigned char)s[i];
        h *= 1099511628211ull;
    }
    return h;
}

static int cache_dir(char* out, size_t cap)
{
    const char* d = getenv("QGT_JIT_CACHE_DIR");
    if (d && *d) {
        snprintf(out, cap, "%s", d);
    } else {
        const char* home = getenv("HOME");
        if (!home || !*home) return -1;
        snprintf(out, cap, "%s/.cache/qgt_gb300_jit", home);
        char parent[1024];
        snprintf(parent, sizeof parent, "%s/.cache", home);
        mkdir(parent, 0700);
    }
    if (mkdir(out, 0700) != 0 && errno != EEXIST) return -1;
    return access(out, W_OK) == 0 ? 0 : -1;
}

static void* read_file(const char* path, size_t* n)
{
    FILE* f = fopen(path, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    void* buf = sz > 0 ? malloc((size_t)sz) : NULL;
    if (buf && fread(buf, 1, (size_t)sz, f) != (size_t)sz) { free(buf); buf = NULL; }
    fclose(f);
    if (buf) *n = (size_t)sz;
    return buf;
}

static void write_file_atomic(const char* path, const void* data, size_t n)
{
    char tmp[1200];
    snprintf(tmp, sizeof tmp, "%s.%d.tmp", path, (int)getpid());
    FILE* f = fopen(tmp, "wb");
    if (!f) return;
    const int ok = fwrite(data, 1, n, f) == n;
    fclose(f);
    if (ok) rename(tmp, path);
    else unlink(tmp);
}

// NVRTC -> cubin bytes (malloc'd)
static int nvrtc_cubin(const char* src, void** cubin, size_t* n)
{
    nvrtcProgram prog;
    nvrtcResult r = nvrtcCreateProgram(&prog, src, "qgt_jit_pass.cu", 0, NULL, NULL);
    if (r != NVRTC_SUCCESS) return qgt_set_error(-6, "jit: nvrtcCreateProgram: %s", nvrtcGetErrorString(r));
    r = nvrtcCompileProgram(prog, JIT_NOPTS, jit_opts);
    if (r != NVRTC_SUCCESS) {
        size_t ls = 0;
        nvrtcGetProgramLogSize(prog, &ls);
        char* log = (char*)malloc(ls + 1);
        if (log) {
            nvrtcGetProgramLog(prog, log);
            log[ls] = 0;
            if (ls > 1500) log[1500] = 0;
        }
        int rc = qgt_set_error(-6, "jit: compile failed: %s: %s", nvrtcGetErrorString(r), log ? log : "");
        free(log);
        nvrtcDestroyProgram(&prog);
        return rc;
    }
    size_t cs = 0;
    r = nvrtcGetCUBINSize(prog, &cs);
    void* buf = (r == NVRTC_SUCCESS && cs) ? malloc(cs) : NULL;
    if (buf) r = nvrtcGetCUBIN(prog, (char*)buf);
    nvrtcDestroyProgram(&prog);
    if (!buf || r != NVRTC_SUCCESS) {
        free(buf);
        return qgt_set_error(-6, "jit: no cubin (%s)", nvrtcGetErrorString(r));
    }
    *cubin = buf;
    *n = cs;
    return 0;
}

static char* full_source(const char* body)
{
    const size_t lp = strlen(jit_prologue), lo = strlen(qgt_pass2_ops_src), lb = strlen(body);
    char* src = (char*)malloc(lp + lo + lb + 2);
    if (!src) return NULL;
    memcpy(src, jit_prologue, lp);
    memcpy(src + lp, qgt_pass2_ops_src, lo);
    src[lp + lo] = '\n';
    memcpy(src + lp + lo + 1, body, lb + 1);
    return src;
}

extern "C" int qgt_jit_nvrtc_check(const char* body, double* seconds)
{
    char* src = full_source(body);
    if (!src) return qgt_set_error(-2, "jit: out of host memory");
    void* cubin = NULL;
    size_t cn = 0;
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    int rc = nvrtc_cubin(src, &cubin, &cn);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    if (seconds) *seconds = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
    free(cubin);
    free(src);
    return rc;
}

static int set_smem(struct qgt_jit_kernel* k, int device)
{
    if (device >= 0 && device < 32 && (k->attr_dev_mask >> device) & 1) return 0;
    cudaError_t e = cudaKernelSetAttributeForDevice(k->kern, cudaFuncAttributeMaxDynamicSharedMemorySize, k->smem, device);
    if (e != cudaSuccess) return qgt_set_error(-6, "jit: shared-memory limit: %s", cudaGetErrorString(e));
    if (device >= 0 && device < 32) k->attr_dev_mask |= 1 << device;
    return 0;
}

extern "C" int qgt_dev_jit_compile(const char* body, const char* kname, int32_t smem, int32_t nthreads, int32_t device,
                                   qgt_jit_kernel_t** out)
{
    *out = NULL;
    if (nthreads != 256 && nthreads != 512 && nthreads != 1024)
        return qgt_set_error(-1, "jit: block of %d threads", nthreads);
    if (cudaSetDevice(device) != cudaSuccess) return qgt_set_error(-6, "jit: device %d", device);
    char* src = full_source(body);
    if (!src) return qgt_set_error(-2, "jit: out of host memory");
    uint64_t key = 1469598103934665603ull;
    key = fnv1a(key, src, strlen(src));
    for (int i = 0; i < JIT_NOPTS; i++) key = fnv1a(key, jit_opts[i], strlen(jit_opts[i]));
    int maj = 0, min = 0;
    nvrtcVersion(&maj, &min);
    char ver[32];
    snprintf(ver, sizeof ver, "nvrtc%d.%d", maj, min);
    key = fnv1a(key, ver, strlen(ver));

    pthread_mutex_lock(&jit_mu);
    for (struct qgt_jit_kernel* k = jit_list; k; k = k->next)
        if (k->key == key) {
            int rc = set_smem(k, device);
            pthread_mutex_unlock(&jit_mu);
            free(src);
            if (!rc) *out = k;
            return rc;
        }
    pthread_mutex_unlock(&jit_mu);

    // disk cache, else the compiler (outside the lock: plans compile their passes in parallel)
    char dir[1024], path[1200];
    const int have_dir = cache_dir(dir, sizeof dir) == 0;
    void* cubin = NULL;
    size_t cn = 0;
    if (have_dir) {
        snprintf(path, sizeof path, "%s/%016llx.cubin", dir, (unsigned long long)key);
        cubin = read_file(path, &cn);
    }
    if (!cubin) {
        struct timespec t0, t1;
        clock_gettime(CLOCK_MONOTONIC, &t0);
        int rc = nvrtc_cubin(src, &cubin, &cn);
        clock_gettime(CLOCK_MONOTONIC, &t1);
        pthread_mutex_lock(&jit_mu);
        jit_seconds += (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
        pthread_mutex_unlock(&jit_mu);
        if (rc) { free(src); return rc; }
        if (have_dir) write_file_atomic(path, cubin, cn);
    }
    free(src);
    struct qgt_jit_kernel* k = (struct qgt_jit_kernel*)calloc(1, sizeof *k);
    if (!k) { free(cubin); return qgt_set_error(-2, "jit: out of host memory"); }
    k->key = key;
    k->smem = smem;
    k->nthreads = nthreads;
    cudaError_t e = cudaLibraryLoadData(&k->lib, cubin, NULL, NULL, 0, NULL, NULL, 0);
    free(cubin);
    if (e == cudaSuccess) e = cudaLibraryGetKernel(&k->kern, k->lib, kname);
    if (e != cudaSuccess) {
        free(k);
        return qgt_set_error(-6, "jit: load %s: %s", kname, cudaGetErrorString(e));
    }
    pthread_mutex_lock(&jit_mu);
    // another thread may have loaded the same image meanwhile: keep one
    for (struct qgt_jit_kernel* o = jit_list; o; o = o->next)
        if (o->key == key) {
            int rc = set_smem(o, device);
            pthread_mutex_unlock(&jit_mu);
            cudaLibraryUnload(k->lib);
            free(k);
            if (!rc) *out = o;
            return rc;
        }
    int rc = set_smem(k, device);
    if (!rc) {
        k->next = jit_list;
        jit_list = k;
        *out = k;
    }
    pthread_mutex_unlock(&jit_mu);
    if (rc) {
        cudaLibraryUnload(k->lib);
        free(k);
    }
    return rc;
}

extern "C" int qgt_dev_jit_launch(const qgt_jit_kernel_t* k, const qgt_dev_pass2_args_t* a, void* stream)
{
    if (a->nentries <= 0) return 0;
    const int64_t ntiles = (int64_t)1 << (a->n - a->tile_bits);
    const int np = a->npoints > 0 ? a->npoints : 1;
    if (a->tile_bits < 13 || a->tile_bits > 14 || a->nentries > 65535 || ntiles > 0x7fffffff || np > 65535)
        return qgt_set_error(-1, "jit: launch shape (%d tile bits, %d entries, %d points)", a->tile_bits, a->nentries, np);
    float2* V = (float2*)a->V;
    long long N = (long long)a->N;
    const int* ents = (const int*)a->entries;
    const float* coef32 = a->coef32;
    unsigned* rowmax = a->rowmax;
    int coef_stride = a->coef_stride;
    long long point_stride = (long long)a->point_stride;
    int rowmax_stride = a->rowmax_stride;
    void* args[] = {&V, &N, &ents, &coef32, &rowmax, &coef_stride, &point_stride, &rowmax_stride};
    dim3 grid((unsigned)ntiles, (unsigned)a->nentries, (unsigned)np);
    cudaError_t e = cudaLaunchKernel((const void*)k->kern, grid, dim3((unsigned)k->nthreads), args, (size_t)k->smem,
                                     (cudaStream_t)stream);
    if (e != cudaSuccess) return qgt_set_error(-6, "jit: launch: %s", cudaGetErrorString(e));
    return 0;
}
