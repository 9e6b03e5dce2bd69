"""The reference-side binding documented in INTEGRATION.md compiles, links
against libperks_gb300.so and runs.

The two C++ blocks of INTEGRATION.md (perks_binding.cpp for the 2D stencils,
perks_binding3d.cpp for the 3D ones) are compiled exactly as they stand there,
with a stand-in for the reference's per-shape config.cuh, together with a
small driver in the role of the reference's jacobi.driver.cpp /
j3d.driver.cpp. The driver declares the templates as the reference's
stencil/2dstencil/common/jacobi_cuda.cuh:6-7 and
stencil/3dstencil/common/jacobi_cuda.cuh:6-7 declare them and calls
jacobi_iterative<double> and j3d_iterative<float> on host arrays read from
files. Building needs no GPU; running is a GPU test, bit-exact against the
oracle."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DOC = os.path.join(ROOT, "INTEGRATION.md")

DRIVER = r'''
#include <cstdio>
#include <cstdlib>
#include <vector>
// as the reference's stencil/2dstencil/common/jacobi_cuda.cuh and
// stencil/3dstencil/common/jacobi_cuda.cuh declare them
template<class REAL>
int jacobi_iterative(REAL*, int, int, REAL*, int, int, int, bool,bool,bool,int,bool);
template<class REAL>
int j3d_iterative(REAL*, int, int, int, REAL*, int, int, int, bool, bool, int, bool, bool getminHeight=false);

template <class T>
static std::vector<T> read_all(const char* path, size_t n) {
  std::vector<T> v(n);
  FILE* f = std::fopen(path, "rb");
  if (!f || std::fread(v.data(), sizeof(T), n, f) != n) std::exit(3);
  std::fclose(f);
  return v;
}
template <class T>
static void write_all(const char* path, const std::vector<T>& v) {
  FILE* f = std::fopen(path, "wb");
  if (!f || std::fwrite(v.data(), sizeof(T), v.size(), f) != v.size()) std::exit(4);
  std::fclose(f);
}

// usage: driver 2d <wy> <wx> <steps> <in> <out>   (double)
//        driver 3d <h> <wy> <wx> <steps> <in> <out>   (float)
int main(int argc, char** argv) {
  if (argc >= 7 && argv[1][0] == '2') {
    const int wy = std::atoi(argv[2]), wx = std::atoi(argv[3]), steps = std::atoi(argv[4]);
    std::vector<double> in = read_all<double>(argv[5], size_t(wy) * wx), out(size_t(wy) * wx);
    const int rc = jacobi_iterative<double>(in.data(), wy, wx, out.data(), 256, 0, steps, false, true, false, 0,
                                            false);
    std::printf("rc=%d\n", rc);
    if (rc != 0) return 1;
    write_all(argv[6], out);
    return 0;
  }
  if (argc >= 8 && argv[1][0] == '3') {
    const int h = std::atoi(argv[2]), wy = std::atoi(argv[3]), wx = std::atoi(argv[4]), steps = std::atoi(argv[5]);
    std::vector<float> in = read_all<float>(argv[6], size_t(h) * wy * wx), out(size_t(h) * wy * wx);
    const int rc = j3d_iterative<float>(in.data(), h, wy, wx, out.data(), 256, 0, steps, true, false, 0, false);
    std::printf("rc=%d\n", rc);
    if (rc != 0) return 1;
    write_all(argv[7], out);
    return 0;
  }
  return 2;
}
'''

# stand-ins for the reference's config.cuh of 2d5pt (HALO 1) and poisson
# (HALO 1 with BOX, TYPE0 and POISSON)
CONFIG_2D = "#define HALO (1)\n"
CONFIG_3D = "#define HALO (1)\n#define BOX\n#define TYPE0\n#define POISSON\n"


def doc_block(name):
    src = open(DOC).read()
    for m in re.finditer(r"```cpp\n(.*?)```", src, re.S):
        if m.group(1).startswith("// " + name):
            return m.group(1)
    raise AssertionError(f"INTEGRATION.md has no C++ block {name}")


@pytest.fixture(scope="module")
def driver(native, tmp_path_factory):
    d = tmp_path_factory.mktemp("binding")
    objs = []
    for name, cfg in (("perks_binding.cpp", CONFIG_2D), ("perks_binding3d.cpp", CONFIG_3D)):
        sub = d / name.replace(".cpp", "")
        sub.mkdir()
        (sub / "config.cuh").write_text(cfg)
        (sub / name).write_text(doc_block(name))
        obj = str(sub / (name + ".o"))
        subprocess.run(["g++", "-std=c++11", "-Wall", "-Werror", "-c", "-I" + os.path.join(ROOT, "include"),
                        "-I" + str(sub), str(sub / name), "-o", obj], check=True)
        objs.append(obj)
    (d / "driver.cpp").write_text(DRIVER)
    lib = native._native.LIB_PATH
    exe = str(d / "driver")
    subprocess.run(["g++", "-std=c++11", "-Wall", "-Werror", str(d / "driver.cpp")] + objs +
                   ["-L" + os.path.dirname(lib), "-lperks_gb300", "-Wl,-rpath," + os.path.dirname(lib), "-o", exe],
                   check=True)
    return exe


def test_binding_compiles_and_links(driver):
    out = subprocess.run(["nm", "-C", driver], capture_output=True, text=True).stdout
    assert "jacobi_iterative<double>" in out and "j3d_iterative<float>" in out


@pytest.mark.gpu
def test_binding_runs_bit_exact(driver, cuda, oracle, tmp_path):
    from test_stencil_gpu import bits_equal
    f = np.random.default_rng(31).random((300, 517))
    f.tofile(tmp_path / "in2")
    r = subprocess.run([driver, "2d", "300", "517", "9", str(tmp_path / "in2"), str(tmp_path / "out2")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    got = np.fromfile(tmp_path / "out2", dtype=np.float64).reshape(f.shape)
    assert bits_equal(got, oracle.stencil("2d5pt", f, 9))
    g = np.random.default_rng(32).random((20, 33, 70)).astype(np.float32)
    g.tofile(tmp_path / "in3")
    r = subprocess.run([driver, "3d", "20", "33", "70", "5", str(tmp_path / "in3"), str(tmp_path / "out3")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    got = np.fromfile(tmp_path / "out3", dtype=np.float32).reshape(g.shape)
    assert bits_equal(got, oracle.stencil("poisson", g, 5))
