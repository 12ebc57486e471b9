/* Bit-exact restatement of the GROG grid-index arithmetic of
 * src/GROG.jl:89-94 (test infrastructure: the oracle for the CUDA kernel).
 *
 *   trj_i = trj * N + 1/2     Float32 * Int -> Float32, then + Float64 -> Float64
 *   k     = round(trj_i)      round-half-to-even
 *   shift = (k - trj_i) * Nr / N   (Float64, evaluated left to right)
 *   idx   = Int(k) + N / 2    (integer division), stored as Int32
 *
 * Compiled without floating-point contraction so no FMA merges the steps.
 * Arrays are column-major (d, n) with d fastest, as in the reference.
 */
#include <math.h>
#include <stdint.h>

void oracle_grog_index(const float *trj, int64_t d, int64_t n, const int64_t *img_shape,
                       int64_t Nr, int32_t *idx, double *shift)
{
    for (int64_t s = 0; s < n; ++s) {
        for (int64_t i = 0; i < d; ++i) {
            const int64_t N = img_shape[i];
            volatile float p = trj[s * d + i] * (float)N;
            volatile double t = (double)p + 0.5;
            double k = nearbyint(t);           /* default rounding mode: ties to even */
            volatile double diff = k - t;
            volatile double num = diff * (double)Nr;
            shift[s * d + i] = num / (double)N;
            idx[s * d + i] = (int32_t)((int64_t)k + N / 2);
        }
    }
}
