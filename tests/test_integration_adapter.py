"""The C++ adapter that INTEGRATION.md shows a maintainer adding to the
reference (the four reference classes as thin functions over one vs_session,
the fused frame call, the batch runner and the serving loop) compiles against
include/vs.h and links against libvs_gb300.so.  The snippets are taken from
the document itself, so the document cannot drift from the header.  The
program then runs on the host: without a GPU session creation reports
VS_ERR_CUDA, with one it succeeds; either way it must link and run."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# names the statement snippets use, declared as parameters of their wrapper
SNIPPET_PARAMS = ("GbScanner& g, const uint16_t* depth_mm_host, vs_session* s0, vs_session* s1, vs_session* s2, "
                  "const uint16_t* f0, const uint16_t* f1, const uint16_t* f2, const vs_config& cfg")


def test_integration_cpp_adapter_compiles_links_and_runs(built, tmp_path):
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if cxx is None:
        pytest.skip("no C++ compiler")
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```cpp\n(.*?)```", doc, flags=re.S)
    assert len(blocks) >= 4, "INTEGRATION.md lost its C++ snippets"
    src = [blocks[0]]  # the adapter: file-scope declarations
    for k, b in enumerate(blocks[1:]):
        src.append("static void snippet_%d(%s) {\n%s}\n" % (k, SNIPPET_PARAMS, b))
    src.append('''
#include <cstdio>
int main() {
  GbScanner g;
  const float origin[3] = {-0.75f, -0.75f, 0.25f};
  const bool ok = g.init(64, 48, 60.f, 60.f, 31.5f, 23.5f, 64, origin, 1.5f / 64, 0.06f, 100.f, 0.01f);
  std::printf("init %d: %s\\n", ok ? 1 : 0, ok ? "ok" : vs_last_error());
  if (!ok && vs_device_count() > 0) return 1;
  return 0;
}
''')
    cpp = tmp_path / "adapter.cpp"
    cpp.write_text("\n".join(src))
    exe = tmp_path / "adapter"
    lib_dir = os.path.join(ROOT, "vcl-volume-scanner_gb300")
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Wno-unused-function", "-I", os.path.join(ROOT, "include"),
                        str(cpp), "-o", str(exe), "-L", lib_dir, "-lvs_gb300", "-Wl,-rpath," + lib_dir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("init ")
