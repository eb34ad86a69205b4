// Test-infrastructure shim, not product code.
//
// The reference includes "../lib/pcg-cpp/include/pcg_random.hpp"
// (src/ncvis.cpp:10), a git submodule (imneme/pcg-cpp, pinned commit unknown)
// that is empty in the reference checkout.  pyarrow vendors the same
// header-only library; this shim forwards to it and exposes its pcg64
// (setseq_xsl_rr_128_64) in the global namespace, as pcg-cpp does.  The build
// recipe passes pyarrow's include directory with -I.
#ifndef ORACLE_SHIM_PCG_RANDOM_HPP
#define ORACLE_SHIM_PCG_RANDOM_HPP

#include <arrow/vendored/pcg/pcg_random.hpp>

using arrow_vendored::pcg64;

#endif
