// CPU stand-in for the wavelet convolution of the reference box-source
// generator -- TEST INFRASTRUCTURE ONLY, linked into the reference program
// built by oracle/build_ref.py, never into the product.
//
// The reference runs this step as a CUDA kernel (cu_con / convolve,
// PSV/psv_clean_double/source/cu_source.cu:2-42) that cannot run without a
// GPU; this file restates its arithmetic so the rest of the reference
// program (Green's functions, wavelets, geometry, file layout) runs on the
// CPU: f2[k] <- sum_j x[j] f2[k-j] over k < n2 (f2 = 0 before sample 0),
// the taps padded with zeros to a multiple of 32 and taken from the last to
// the first, one fused multiply-add each (the kernel's "sum += f1*s" with
// the compiler's default contraction).
#include <cmath>
#include <vector>

void cu_con(int n1, double *x, int n2, double *f2)
{
    const int ntap = ((n1 - 1) / 32 + 1) * 32;
    std::vector<double> tap(ntap, 0.0), in(f2, f2 + n2);
    for (int j = 0; j < n1; ++j) tap[j] = x[j];
    for (int k = 0; k < n2; ++k) {
        double acc = 0.0;
        for (int j = ntap - 1; j >= 0; --j) acc = std::fma(tap[j], k - j >= 0 ? in[k - j] : 0.0, acc);
        f2[k] = acc;
    }
}
