// capi.cu -- the extern "C" boundary (include/sankhya_gb300.h).
//
// Every entry point catches everything: EngineError becomes its code, std::bad_alloc becomes
// SANKHYA_GB300_ERROR_MEMORY and anything else SANKHYA_GB300_ERROR_INTERNAL, with the text in
// a thread-local last-error string -- the reference C API's rules (src/api/c_api.cpp:39,
// 134-150).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "batch_engine.hpp"
#include "engine.hpp"
#include "qp_engine.hpp"
#include "sankhya_gb300.h"

struct sankhya_gb300_pdhg {
  sgb::Engine* engine;
};

struct sankhya_gb300_batch {
  sgb::BatchEngine* engine;
};

struct sankhya_gb300_qp {
  sgb::QpEngine* engine;
};

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& message) {
  g_last_error = message;
  return code;
}

template <typename F>
int guarded(F&& body) {
  try {
    body();
    g_last_error.clear();
    return SANKHYA_GB300_OK;
  } catch (const sgb::EngineError& e) {
    return fail(e.code, e.message);
  } catch (const std::bad_alloc&) {
    return fail(SANKHYA_GB300_ERROR_MEMORY, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(SANKHYA_GB300_ERROR_INTERNAL, e.what());
  } catch (...) {
    return fail(SANKHYA_GB300_ERROR_INTERNAL, "unknown exception");
  }
}

}  // namespace

extern "C" {

SGB_API const char* sankhya_gb300_last_error(void) { return g_last_error.c_str(); }

SGB_API int sankhya_gb300_device_available(char* description, int32_t capacity) {
  int count = 0;
  const cudaError_t err = cudaGetDeviceCount(&count);
  if (err != cudaSuccess || count <= 0) {
    cudaGetLastError();
    const std::string why = err != cudaSuccess ? std::string("no device: ") + cudaGetErrorString(err)
                                               : std::string("no device: none present");
    if (description != nullptr && capacity > 0) std::snprintf(description, capacity, "%s", why.c_str());
    return fail(SANKHYA_GB300_ERROR_DEVICE, why);
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, 0) != cudaSuccess) {
    return fail(SANKHYA_GB300_ERROR_DEVICE, "cudaGetDeviceProperties failed");
  }
  if (description != nullptr && capacity > 0) {
    std::snprintf(description, capacity, "%s (compute %d.%d, %zu MiB VRAM)", prop.name, prop.major,
                  prop.minor, static_cast<size_t>(prop.totalGlobalMem >> 20));
  }
  g_last_error.clear();
  return SANKHYA_GB300_OK;
}

SGB_API int sankhya_gb300_device_free_memory(size_t* free_bytes, size_t* total_bytes) {
  size_t f = 0, t = 0;
  const cudaError_t err = cudaMemGetInfo(&f, &t);
  if (err != cudaSuccess) {
    cudaGetLastError();
    return fail(SANKHYA_GB300_ERROR_DEVICE, cudaGetErrorString(err));
  }
  if (free_bytes) *free_bytes = f;
  if (total_bytes) *total_bytes = t;
  return SANKHYA_GB300_OK;
}

SGB_API int sankhya_gb300_device_compute_capability(int32_t* major, int32_t* minor) {
  int dev = 0;
  cudaDeviceProp prop;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
    cudaGetLastError();
    return fail(SANKHYA_GB300_ERROR_DEVICE, "no CUDA device");
  }
  if (major) *major = prop.major;
  if (minor) *minor = prop.minor;
  return SANKHYA_GB300_OK;
}

SGB_API size_t sankhya_gb300_estimate_memory(int32_t rows, int32_t cols, int64_t nonzeros,
                                             int32_t precision) {
  return sgb::estimate_memory(rows, cols, nonzeros, precision);
}

SGB_API int sankhya_gb300_pdhg_create(int32_t device, sankhya_gb300_pdhg** out) {
  if (out == nullptr) return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null output handle");
  *out = nullptr;
  return guarded([&] {
    sgb::Engine* e = new sgb::Engine(device);
    *out = new sankhya_gb300_pdhg{e};
  });
}

SGB_API int sankhya_gb300_pdhg_destroy(sankhya_gb300_pdhg* engine) {
  if (engine == nullptr) return SANKHYA_GB300_OK;
  return guarded([&] {
    delete engine->engine;
    delete engine;
  });
}

SGB_API int sankhya_gb300_pdhg_load(sankhya_gb300_pdhg* engine, const sankhya_gb300_lp* lp) {
  if (engine == nullptr || lp == nullptr) return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null argument");
  return guarded([&] { engine->engine->load(*lp); });
}

SGB_API int sankhya_gb300_pdhg_solve(sankhya_gb300_pdhg* engine,
                                     const sankhya_gb300_params* params,
                                     sankhya_gb300_result* result) {
  if (engine == nullptr || params == nullptr || result == nullptr) {
    return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null argument");
  }
  if (!(params->tolerance >= 0.0)) return fail(SANKHYA_GB300_ERROR_OPTION, "pdhg_tolerance must be >= 0");
  return guarded([&] { engine->engine->solve(*params, result); });
}

SGB_API int sankhya_gb300_pdhg_solution(sankhya_gb300_pdhg* engine, double* col_value,
                                        double* col_dual, double* row_dual) {
  if (engine == nullptr) return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null engine");
  return guarded([&] { engine->engine->solution(col_value, col_dual, row_dual); });
}

SGB_API int sankhya_gb300_pdhg_scaling(sankhya_gb300_pdhg* engine, int64_t random_seed,
                                       double* row_scale, double* col_scale,
                                       double* scaled_values, double* spectral_norm) {
  if (engine == nullptr) return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null engine");
  return guarded([&] {
    engine->engine->scaling(random_seed, row_scale, col_scale, scaled_values, spectral_norm);
  });
}

SGB_API int sankhya_gb300_pdhg_spmv(sankhya_gb300_pdhg* engine, int32_t op, int32_t scaled,
                                    const double* in, double* out) {
  if (engine == nullptr || in == nullptr || out == nullptr || (op != 0 && op != 1)) {
    return fail(SANKHYA_GB300_ERROR_ARGUMENT, "bad spmv arguments");
  }
  return guarded([&] { engine->engine->spmv(op, scaled, in, out); });
}

SGB_API int sankhya_gb300_pdhg_spmv_noalloc(sankhya_gb300_pdhg* engine, int32_t op,
                                            int32_t scaled, const double* device_in,
                                            double* device_out, void* stream) {
  if (engine == nullptr || engine->engine == nullptr) {
    return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null engine");
  }
  return guarded([&] {
    engine->engine->spmv_noalloc(op, scaled, device_in, device_out,
                                 static_cast<cudaStream_t>(stream));
  });
}

SGB_API int sankhya_gb300_pdhg_time_kernels(sankhya_gb300_pdhg* engine, int32_t reps,
                                            double* ms) {
  if (engine == nullptr || ms == nullptr || reps <= 0) {
    return fail(SANKHYA_GB300_ERROR_ARGUMENT, "bad time_kernels arguments");
  }
  return guarded([&] { engine->engine->time_kernels(reps, ms); });
}

SGB_API int sankhya_gb300_batch_create(int32_t device, sankhya_gb300_batch** out) {
  if (out == nullptr) return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null output handle");
  *out = nullptr;
  return guarded([&] {
    sgb::BatchEngine* e = new sgb::BatchEngine(device);
    *out = new sankhya_gb300_batch{e};
  });
}

SGB_API int sankhya_gb300_batch_destroy(sankhya_gb300_batch* batch) {
  if (batch == nullptr) return SANKHYA_GB300_OK;
  return guarded([&] {
    delete batch->engine;
    delete batch;
  });
}

SGB_API int sankhya_gb300_batch_load(sankhya_gb300_batch* batch, int32_t count,
                                     const sankhya_gb300_lp* lps) {
  if (batch == nullptr || lps == nullptr || count <= 0) {
    return fail(SANKHYA_GB300_ERROR_ARGUMENT, "bad batch_load arguments");
  }
  return guarded([&] { batch->engine->load(count, lps); });
}

SGB_API int sankhya_gb300_batch_solve(sankhya_gb300_batch* batch,
                                      const sankhya_gb300_params* params,
                                      sankhya_gb300_batch_item* items, double* device_seconds) {
  if (batch == nullptr || params == nullptr || items == nullptr) {
    return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null argument");
  }
  return guarded([&] { batch->engine->solve(*params, items, device_seconds); });
}

SGB_API int sankhya_gb300_batch_schedule(sankhya_gb300_batch* batch, int32_t lanes,
                                         int32_t threads) {
  if (batch == nullptr) return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null batch");
  return guarded([&] { batch->engine->set_schedule(lanes, threads); });
}

SGB_API int sankhya_gb300_batch_last_schedule(sankhya_gb300_batch* batch, int32_t* lanes,
                                              int32_t* threads, double* tune_seconds) {
  if (batch == nullptr) return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null batch");
  return guarded([&] {
    int l = 0, t = 0;
    batch->engine->last_schedule(&l, &t, tune_seconds);
    if (lanes != nullptr) *lanes = l;
    if (threads != nullptr) *threads = t;
  });
}

SGB_API int sankhya_gb300_batch_solution(sankhya_gb300_batch* batch, int32_t index,
                                         double* col_value, double* col_dual,
                                         double* row_dual) {
  if (batch == nullptr) return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null batch");
  return guarded([&] { batch->engine->solution(index, col_value, col_dual, row_dual); });
}

SGB_API int sankhya_gb300_batch_set_point(sankhya_gb300_batch* batch, int32_t index,
                                          const double* col_value, const double* col_dual,
                                          const double* row_dual) {
  if (batch == nullptr) return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null batch");
  return guarded([&] { batch->engine->set_point(index, col_value, col_dual, row_dual); });
}

SGB_API int sankhya_gb300_batch_ray(sankhya_gb300_batch* batch, int32_t index, double* ray) {
  if (batch == nullptr) return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null batch");
  return guarded([&] { batch->engine->ray(index, ray); });
}

SGB_API int sankhya_gb300_batch_adjoint(sankhya_gb300_batch* batch,
                                        const double* const* dl_dx, const double* const* dl_dy,
                                        const double* dl_df, double* const* dl_dc,
                                        double* const* dl_drl, double* const* dl_dru,
                                        double* const* dl_dl, double* const* dl_du,
                                        sankhya_gb300_adjoint_info* info) {
  if (batch == nullptr) return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null batch");
  return guarded([&] {
    batch->engine->adjoint(dl_dx, dl_dy, dl_df, dl_dc, dl_drl, dl_dru, dl_dl, dl_du, info);
  });
}

SGB_API int sankhya_gb300_batch_polish(sankhya_gb300_batch* batch,
                                       sankhya_gb300_batch_item* items,
                                       sankhya_gb300_adjoint_info* info) {
  if (batch == nullptr) return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null batch");
  return guarded([&] { batch->engine->polish(items, info); });
}

// ---- Convex QP ----

SGB_API int sankhya_gb300_qp_create(int32_t device, sankhya_gb300_qp** out) {
  if (out == nullptr) return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null output handle");
  *out = nullptr;
  return guarded([&] {
    sgb::QpEngine* e = new sgb::QpEngine(device);
    *out = new sankhya_gb300_qp{e};
  });
}

SGB_API int sankhya_gb300_qp_destroy(sankhya_gb300_qp* engine) {
  if (engine == nullptr) return SANKHYA_GB300_OK;
  return guarded([&] {
    delete engine->engine;
    delete engine;
  });
}

SGB_API int sankhya_gb300_qp_load(sankhya_gb300_qp* engine,
                                  const sankhya_gb300_qp_problem* problem) {
  if (engine == nullptr || problem == nullptr) {
    return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null engine or QP");
  }
  return guarded([&] { engine->engine->load(*problem); });
}

SGB_API int sankhya_gb300_qp_solve(sankhya_gb300_qp* engine,
                                   const sankhya_gb300_qp_params* params,
                                   sankhya_gb300_qp_result* result) {
  if (engine == nullptr || params == nullptr || result == nullptr) {
    return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null engine, parameters or result");
  }
  return guarded([&] { engine->engine->solve(*params, result); });
}

SGB_API int sankhya_gb300_qp_solution(sankhya_gb300_qp* engine, double* col_value,
                                      double* col_dual, double* row_dual) {
  if (engine == nullptr) return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null engine");
  return guarded([&] { engine->engine->solution(col_value, col_dual, row_dual); });
}

SGB_API int sankhya_gb300_qp_time_kernels(sankhya_gb300_qp* engine, int32_t reps, double* ms) {
  if (engine == nullptr || ms == nullptr) {
    return fail(SANKHYA_GB300_ERROR_ARGUMENT, "null engine or output");
  }
  return guarded([&] { engine->engine->time_kernels(reps, ms); });
}

}  // extern "C"
