// Definition of the opaque C handle, shared by the translation units that implement the C
// interface (capi.cu, noalloc.cu).
#pragma once

#include <memory>
#include <string>

#include "framework/context.h"

struct pimc_ctx {
    std::unique_ptr<pimc::Context> c;
    std::string err;
};
