// Empty stand-in for the reference's vendored copy of Eigen's unsupported NNLS
// module (nnls/interface/eigen_nnls.h). multifit_cpu/src/PulseChiSqSNNLS.cpp
// includes it but calls none of it (its Eigen::NNLS call is commented out), and
// its templates need parts of Eigen the oracle's shim does not provide.
// TEST INFRASTRUCTURE ONLY (the reference-DoFit pin, oracle/ref_dofit_driver.cpp).
#pragma once
