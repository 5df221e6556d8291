// qgt_noalloc_solve.cu -- (A + lambda I) x = g by FP64 Cholesky with every
// device buffer taken from one file-scope static array, so that a call makes
// no device allocation of its own.
//
// Who needs it: callers whose device memory is fully owned by another
// allocator (a framework's caching pool holding the rest of HBM, where a new
// cudaMalloc can fail or fragment it), and callers that solve small systems
// in a tight optimiser loop and cannot take the device-wide synchronisation
// that cudaFree performs on every call of the allocating entry point.
//
// Scratch: QGT_NOALLOC_SOLVE_MAX_P (512) sets the size; the array holds a copy
// of A, the Cholesky factor, g, x and a two-word status, 2 P^2 + 2 P + 2
// doubles at P = 512 (about 4.2 MB), fixed when the library loads.  No word of
// it needs to start at zero: the kernel rebuilds the factor from A on every
// attempt, writes each y_i / x_i before it reads it, and writes the status
// last; the host copies A and g in before the launch.
//
// Set-up: the first call on each device, with that device current, looks up
// the array's device address with cudaGetSymbolAddress (which may load this
// file's module on that device) and keeps it for later calls.  Make that
// first call on a device before any stream capture begins there.
//
// Concurrency: all calls on one device share the one array.  Two calls that
// overlap in time on the same device (two host threads, say) race on it and
// can return each other's results; serialise them.
#include <cuda_runtime.h>
#include <mutex>

#include "../qgt_internal.h"
#include "qgt_gb300.h"

#define NA_MAXP QGT_NOALLOC_SOLVE_MAX_P
#define NA_MAX_DEVICES 64

// [A: MAXP^2][L: MAXP^2][g: MAXP][x: MAXP][status: 2]; every offset is a
// multiple of 512 doubles, so each piece keeps the array's 256-byte alignment
static __device__ __align__(256) double noalloc_scratch[2 * NA_MAXP * NA_MAXP + 2 * NA_MAXP + 2];

static std::mutex na_mutex;
static double* na_base[NA_MAX_DEVICES];

static int na_fail(cudaError_t e, const char* what)
{
    return qgt_set_error(-6, "qgt_cholesky_solve_f64_noalloc: %s: %s", what, cudaGetErrorString(e));
}

// device address of the scratch on the current device, looked up once
static int na_scratch(double** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return na_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= NA_MAX_DEVICES)
        return qgt_set_error(-1, "qgt_cholesky_solve_f64_noalloc: device %d beyond %d", dev, NA_MAX_DEVICES);
    std::lock_guard<std::mutex> lock(na_mutex);
    if (!na_base[dev]) {
        double* ptr = nullptr;
        e = cudaGetSymbolAddress((void**)&ptr, noalloc_scratch);
        if (e != cudaSuccess) return na_fail(e, "cudaGetSymbolAddress");
        na_base[dev] = ptr;
    }
    *out = na_base[dev];
    return 0;
}

extern "C" int qgt_cholesky_solve_f64_noalloc(const double* A, const double* g, double lambda, int32_t P, double* x,
                                              double* lambda_used)
{
    if (!A || !g || !x || P <= 0) return qgt_set_error(-1, "qgt_cholesky_solve_f64_noalloc: bad argument");
    if (P > NA_MAXP)
        return qgt_set_error(-1, "qgt_cholesky_solve_f64_noalloc: P = %d exceeds the static scratch maximum %d "
                             "(use qgt_cholesky_solve_f64)", (int)P, NA_MAXP);
    double* base = nullptr;
    int rc = na_scratch(&base);
    if (rc) return rc;
    double* A_d = base;
    double* L_d = base + (size_t)NA_MAXP * NA_MAXP;
    double* g_d = base + (size_t)2 * NA_MAXP * NA_MAXP;
    double* x_d = g_d + NA_MAXP;
    double* st_d = x_d + NA_MAXP;
    // legacy default stream throughout: each copy is ordered after the last
    cudaError_t e = cudaMemcpy(A_d, A, sizeof(double) * (size_t)P * P, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return na_fail(e, "copy of A");
    e = cudaMemcpy(g_d, g, sizeof(double) * (size_t)P, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return na_fail(e, "copy of g");
    rc = qgt_dev_cholesky(A_d, 0, g_d, P, lambda, L_d, x_d, st_d, nullptr);
    if (rc) return rc;
    double st[2] = {0, 0};
    e = cudaMemcpy(x, x_d, sizeof(double) * (size_t)P, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return na_fail(e, "copy of x");
    e = cudaMemcpy(st, st_d, sizeof st, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return na_fail(e, "copy of the status");
    if (lambda_used) *lambda_used = st[1];
    if ((int)st[0]) return qgt_set_error((int)st[0], "cholesky: matrix not positive definite after lambda retries");
    return 0;
}
