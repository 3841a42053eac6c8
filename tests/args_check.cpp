// Host check of the device-buffer argument rules (rocflu_gb300/csrc/args.h)
// that rflu_gpu_residual_static applies before it launches anything: every
// branch with a context on device 0 and on device 3.  Built and run by
// tests/test_args_cpu.py.
#include <cstdio>
#include <cstring>
#include <initializer_list>

#include "args.h"

int main() {
  using rflu::ArgMem;
  using rflu::deviceArgProblem;
  int fails = 0;
  auto expect = [&](bool ok, const char *what) {
    if (!ok) {
      std::printf("FAIL %s\n", what);
      ++fails;
    }
  };
  for (int ctx : {0, 3}) {
    expect(deviceArgProblem(ArgMem::Device, ctx, ctx, ctx) == nullptr, "device buffer on the context's device");
    expect(deviceArgProblem(ArgMem::Managed, -1, ctx, ctx) == nullptr, "managed buffer");
    expect(deviceArgProblem(ArgMem::Managed, ctx + 1, ctx, ctx) == nullptr, "managed buffer allocated elsewhere");
    const char *peer = deviceArgProblem(ArgMem::Device, ctx + 1, ctx, ctx);
    expect(peer && std::strstr(peer, "another device"), "device buffer on another device");
    const char *host = deviceArgProblem(ArgMem::Host, -1, ctx, ctx);
    expect(host && std::strstr(host, "device (or managed) memory"), "pinned host buffer");
    const char *unk = deviceArgProblem(ArgMem::Unknown, -1, ctx, ctx);
    expect(unk && std::strstr(unk, "device (or managed) memory"), "pageable host buffer");
    const char *cur = deviceArgProblem(ArgMem::Device, ctx, ctx, ctx + 1);
    expect(cur && std::strstr(cur, "current device"), "another device current");
    const char *cur2 = deviceArgProblem(ArgMem::Managed, -1, ctx, ctx + 1);
    expect(cur2 && std::strstr(cur2, "current device"), "another device current, managed buffer");
  }
  std::printf(fails ? "failed\n" : "ok\n");
  return fails ? 1 : 0;
}
