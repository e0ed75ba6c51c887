/*
 * game_gpu_numerics: runs one of the mixed path's hand-made FP64 / FP32
 * primitives (kernels.cuh: rcp_nr, to_float, to_double, the double-float
 * helpers of the column solvers) over a host array, next to the CUDA
 * operation it stands for, so that a test can compare the two bit for bit
 * or bound their difference.  Host-in/host-out; needs no context.
 *
 * op  input   output  computes
 *  0  double  double  rcp_nr<1>(x)          (one Newton step on rcp.approx)
 *  1  double  double  rcp_nr<2>(x)
 *  2  double  double  1.0 / x               (IEEE division)
 *  3  double  float   to_float(x)           (integer-pipe rounding)
 *  4  double  float   __double2float_rn(x)
 *  5  float   double  to_double(x)          (integer-pipe widening)
 *  6  float   double  (double)x
 *  7  double  double  df_from_double(x) -> back to double: hi + lo
 *                     (the double-float split and its exact join)
 *  8  double  double  df_rcp(x) joined      (double-float reciprocal)
 *  9  double  double  df_mul(df(x), df(y)) joined, y = in[n + i]
 * 10  double  double  df_add(df(x), df(y)) joined, y = in[n + i]
 */
#include <cuda_runtime.h>

#include <string>

#include "context.h"
#include "dfloat.cuh"
#include "game_gb300.h"
#include "kernels.cuh"

namespace game {
namespace {

__global__ void k_numerics(int op, const void *in, void *out, long long n)
{
    const long long i = gtid();
    if (i >= n) return;
    const double *xd = (const double *)in;
    const float *xf = (const float *)in;
    double *od = (double *)out;
    float *of = (float *)out;
    switch (op) {
    case 0: od[i] = rcp_nr<1>(xd[i]); break;
    case 1: od[i] = rcp_nr<2>(xd[i]); break;
    case 2: od[i] = 1.0 / xd[i]; break;
    case 3: of[i] = to_float(xd[i]); break;
    case 4: of[i] = __double2float_rn(xd[i]); break;
    case 5: od[i] = to_double(xf[i]); break;
    case 6: od[i] = (double)xf[i]; break;
    case 7: od[i] = df_to_double(df_from_double(xd[i])); break;
    case 8: od[i] = df_to_double(df_rcp(df_from_double(xd[i]))); break;
    case 9: od[i] = df_to_double(df_mul(df_from_double(xd[i]), df_from_double(xd[n + i]))); break;
    case 10: od[i] = df_to_double(df_add(df_from_double(xd[i]), df_from_double(xd[n + i]))); break;
    default: break;
    }
}

}  // namespace
}  // namespace game

using namespace game;

extern "C" int game_gpu_numerics(int op, const void *in, void *out, long long n)
{
    if (op < 0 || op > 10) return fail("game_gpu_numerics: unknown op " + std::to_string(op));
    if (n < 0) return fail("game_gpu_numerics: negative length");
    if (n == 0) return 0;
    if (!in || !out) return fail("game_gpu_numerics: null pointer");
    const size_t in_elem = (op == 5 || op == 6) ? sizeof(float) : sizeof(double);
    const size_t out_elem = (op == 3 || op == 4) ? sizeof(float) : sizeof(double);
    const size_t in_bytes = in_elem * (size_t)n * (op >= 9 ? 2 : 1), out_bytes = out_elem * (size_t)n;
    void *din = nullptr, *dout = nullptr;
    CK(cudaMalloc(&din, in_bytes));
    cudaError_t e = cudaMalloc(&dout, out_bytes);
    if (e == cudaSuccess) e = cudaMemcpy(din, in, in_bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_numerics<<<(unsigned)((n + 255) / 256), 256>>>(op, din, dout, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, out_bytes, cudaMemcpyDeviceToHost);
    cudaFree(din);
    if (dout) cudaFree(dout);
    if (e != cudaSuccess) return fail(std::string("game_gpu_numerics: ") + cudaGetErrorString(e));
    return 0;
}
