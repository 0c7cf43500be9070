#include "context.hpp"
extern "C" int bn_forward(bn_context* ctx, const bn_adjoint_desc*, const float*, const float*, float*) { return ctx ? ctx->fail(BN_ERR_UNSUPPORTED, "adjoint not built") : BN_ERR_INVALID_ARG; }
extern "C" int bn_backward(bn_context* ctx, const bn_adjoint_desc*, const float*, const float*, const float*, double*, double*) { return ctx ? ctx->fail(BN_ERR_UNSUPPORTED, "adjoint not built") : BN_ERR_INVALID_ARG; }
