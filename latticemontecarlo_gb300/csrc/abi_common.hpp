// Error handling shared by the C ABI translation units: C++ exceptions inside,
// int status codes and a per-thread message (lmc_last_error) across the ABI.
#pragma once

#include <cuda_runtime.h>

#include <ios>
#include <stdexcept>
#include <string>

#include "../../include/lmc_gb300.h"

namespace lmc::abi {

inline thread_local std::string g_error;

struct LmcError : std::runtime_error {
  int code;
  LmcError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void CudaCheck(cudaError_t err, const char *what) {
  if (err != cudaSuccess) throw LmcError(LMC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(err));
}

inline void Require(bool ok, int code, const std::string &msg) {
  if (!ok) throw LmcError(code, msg);
}

// Runs f; maps exceptions to the reference's error classes (LmcError carries its code).
template <typename F>
int Guard(F &&f) {
  try {
    f();
    return LMC_OK;
  } catch (const LmcError &e) {
    g_error = e.what();
    return e.code;
  } catch (const std::out_of_range &e) {
    g_error = e.what();
    return LMC_ERR_OUT_OF_RANGE;
  } catch (const std::ios_base::failure &e) {
    g_error = e.what();
    return LMC_ERR_IO;
  } catch (const std::invalid_argument &e) {
    g_error = e.what();
    return LMC_ERR_INVALID_ARGUMENT;
  } catch (const std::exception &e) {
    g_error = e.what();
    return LMC_ERR_INVALID_ARGUMENT;
  }
}

}  // namespace lmc::abi
