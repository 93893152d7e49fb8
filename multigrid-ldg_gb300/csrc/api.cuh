// api.cuh -- try/catch wrapper that maps internal errors to C status codes.
#pragma once

#include <new>

#include "internal.cuh"

#define MG_API_BEGIN(ctxp)                                          \
    mgldg_ctx* api_ctx_ = (ctxp);                                   \
    try {                                                           \
        if (!api_ctx_) return MGLDG_ERR_ARG;                        \
        MG_CHECK_CUDA(cudaSetDevice(api_ctx_->device));

#define MG_API_END                                                  \
    return MGLDG_OK;                                                \
    }                                                               \
    catch (const ::mg::Error& e) {                                  \
        if (api_ctx_) api_ctx_->err = e.what();                     \
        return e.code;                                              \
    }                                                               \
    catch (const std::bad_alloc&) {                                 \
        if (api_ctx_) api_ctx_->err = "host allocation failed";     \
        return MGLDG_ERR_NOMEM;                                     \
    }                                                               \
    catch (const std::exception& e) {                               \
        if (api_ctx_) api_ctx_->err = e.what();                     \
        return MGLDG_ERR_ARG;                                       \
    }
