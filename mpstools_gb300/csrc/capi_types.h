// Handle types and error plumbing shared by the C-ABI translation units (capi.cpp, tebd.cpp).
#pragma once
#include "host_ops.h"

struct mpsg_ctx_s {
  std::shared_ptr<mpsg::Ctx> c;  // tensors, plans and engines hold further references
};
struct mpsg_tensor_s {
  mpsg::TensorP t;
};

#define API_BEGIN try {
#define API_END                                  \
  }                                              \
  catch (const mpsg::Err& ex) {                  \
    mpsg::g_last_error = ex.what();              \
    return (mpsg_status)ex.code;                 \
  }                                              \
  catch (const std::exception& ex) {             \
    mpsg::g_last_error = ex.what();              \
    return MPSG_ERR_ARG;                         \
  }                                              \
  return MPSG_OK;

static inline mpsg::Ctx* C(mpsg_ctx c) {
  MPSG_CHECK(c && c->c, "null context");
  return c->c.get();
}
static inline const mpsg::Tensor& T(mpsg_tensor t) {
  MPSG_CHECK(t && t->t, "null tensor");
  return *t->t;
}
static inline mpsg_tensor wrap(mpsg::TensorP t) {
  mpsg_tensor w = new mpsg_tensor_s;
  w->t = t;
  return w;
}
