// Definition of the opaque C handle, shared by the translation units that implement the C
// interface (capi.cu, noalloc.cu).
#pragma once

#include <memory>
#include <string>

#include "framework/context.h"

namespace pimc {
/// Loads the no-allocation entry point's module (its fixed scratch array) and every kernel that
/// entry point launches on `device`, so that its calls allocate nothing (noalloc.cu).
void NoAllocPrepare(int device);
}  // namespace pimc

struct pimc_ctx {
    std::unique_ptr<pimc::Context> c;
    std::string err;
};
