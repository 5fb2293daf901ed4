// Definitions shared by the translation units of the C-ABI (mf_capi.cu,
// mf_capi_solvers.cu): the opaque handle types of include/mfgpu.h and the
// exception-to-status wrapper.
#pragma once

#include <algorithm>
#include <atomic>
#include <cstring>
#include <string>

#include "../../include/mfgpu.h"
#include "mf_drivers.h"

using namespace mfgpu;

struct mfgpu_context
{
  std::unique_ptr<Context> c;
  std::atomic<int>         live{0}; // operators and drivers created on this context
};

struct mfgpu_operator
{
  std::unique_ptr<Operator> op;
  mfgpu_context            *ctx = nullptr;
  DevBuf                    hsrc, hdst; // device staging for the host-buffer vmult
  HostPipe                  pipe;       // streams of the overlapped host-buffer vmult
};

struct mfgpu_solid
{
  std::unique_ptr<SolidDriver> d;
  mfgpu_context               *ctx = nullptr;
};

struct mfgpu_heat
{
  std::unique_ptr<HeatDriver> d;
  mfgpu_context              *ctx = nullptr;
};



template <typename F>
inline int
guarded(F &&f)
{
  try
    {
      f();
      return MFGPU_OK;
    }
  catch (const Error &e)
    {
      mfgpu::set_last_error(e.what());
      return e.code;
    }
  catch (const std::exception &e)
    {
      mfgpu::set_last_error(e.what());
      return MFGPU_ERR_ARG;
    }
  catch (...)
    {
      mfgpu::set_last_error("unknown exception");
      return MFGPU_ERR_ARG;
    }
}

// copy a text result into a caller's buffer (NUL-terminated, truncated)
inline void
copy_text(const std::string &t, char *buf, size_t len)
{
  if (len == 0)
    throw Error(ERR_ARG, "buffer length 0");
  const size_t k = std::min(t.size(), len - 1);
  std::memcpy(buf, t.data(), k);
  buf[k] = '\0';
}

inline void
need(const void *p, const char *what)
{
  if (!p)
    throw Error(ERR_ARG, std::string("null argument: ") + what);
}

