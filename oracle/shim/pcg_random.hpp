// Forwards to a copy of O'Neill's pcg-cpp (the one vendored by pyarrow in this
// image), which the reference includes as <pcg_random.hpp>.  The include path
// is set by oracle/Makefile.ref.
#pragma once
#include <arrow/vendored/pcg/pcg_random.hpp>
using namespace arrow_vendored;
