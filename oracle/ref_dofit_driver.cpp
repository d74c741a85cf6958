// Thin C driver around the reference's own multifit_cpu fit: the sources
// multifit_cpu/src/PulseChiSqSNNLS.cpp (DoFit, Minimize, updateCov, NNLS,
// ComputeChiSq, ComputeApproxUncertainty) and nnls/src/inplace_fnnls.cu
// (inplace_fnnls), included here unmodified from the reference tree and
// compiled by oracle/build_oracle.py into oracle/_ref/libref_dofit.so.
// TEST INFRASTRUCTURE ONLY: the tests use it to pin the oracle's restatement
// of the outer fit (the layer that needs Eigen) against the reference's own
// control flow.
//
// Eigen, which the reference includes but does not vendor, is replaced by
// the small API shim in oracle/eigen_shim/ (its arithmetic is the oracle's
// canonical order); the vendored Eigen NNLS module, which the fit includes
// but never calls, by an empty header (oracle/eigen_shim_stubs/).

#include "multifit_cpu/src/PulseChiSqSNNLS.cpp"
#include "nnls/src/inplace_fnnls.cu"

extern "C" {

// n channels of N = 10 samples (row-major [n][10]) sharing one condition set:
// samplecor (10 x 10, column-major), bxs (K values), fullpulse (19) and
// fullpulsecov (19 x 19, column-major). For each channel one PulseChiSqSNNLS
// object runs DoFit; outputs X() (K per channel), ChiSq(), the in-time entry
// of Errors() (0 when errors are off) and DoFit's return value.
int ref_dofit_batch(long n, int K, const double* samples, const double* samplecor, const double* pederr,
                    const signed char* bxs, const double* fullpulse, const double* fullpulsecov, int compute_errors,
                    double* amplitudes, double* chi2, double* errors, int* ok) {
  if (K < 1 || K > 10) return 1;
  SampleMatrix cor;
  for (int j = 0; j < 10; ++j)
    for (int i = 0; i < 10; ++i) cor(i, j) = samplecor[i + 10 * j];
  BXVector bx = BXVector::Zero(K);
  int intime = -1;
  for (int k = 0; k < K; ++k) {
    bx.coeffRef(k) = char(bxs[k]);
    if (intime < 0 && bxs[k] == 0) intime = k;
  }
  FullSampleVector fp;
  for (int i = 0; i < 19; ++i) fp(i) = fullpulse[i];
  FullSampleMatrix fpc;
  for (int j = 0; j < 19; ++j)
    for (int i = 0; i < 19; ++i) fpc(i, j) = fullpulsecov ? fullpulsecov[i + 19 * j] : 0.;
  for (long c = 0; c < n; ++c) {
    SampleVector s;
    for (int i = 0; i < 10; ++i) s(i) = samples[c * 10 + i];
    PulseChiSqSNNLS fit;
    if (!compute_errors) fit.disableErrorCalculation();
    ok[c] = fit.DoFit(s, cor, pederr[c], bx, fp, fpc) ? 1 : 0;
    for (int k = 0; k < K; ++k) amplitudes[c * K + k] = fit.X().coeff(k);
    chi2[c] = fit.ChiSq();
    errors[c] = (compute_errors && intime >= 0) ? fit.Errors().coeff(intime) : 0.;
  }
  return 0;
}

}  // extern "C"
