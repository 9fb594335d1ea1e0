import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def lib():
    from symx_gb300 import build, capi
    build.build()
    return capi.load()


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    d = os.path.join(ROOT, "tests", "golden")

    def load(name):
        return np.load(os.path.join(d, name + ".npz"), allow_pickle=False)

    return load


@pytest.fixture(scope="session")
def compiled_test(lib):
    """tests/cpp/test_compiled.cpp built against the library (C++ Compiled<T> API)."""
    import subprocess

    from symx_gb300.build import cuda_home

    libdir = os.path.join(ROOT, "symx_gb300", "_build")
    exe = os.path.join(libdir, "test_compiled")
    cuda = cuda_home()
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(cuda, "include"),
                    os.path.join(ROOT, "tests", "cpp", "test_compiled.cpp"), "-o", exe, "-L" + libdir, "-lsymxg",
                    "-Wl,-rpath," + libdir, "-L" + os.path.join(cuda, "lib64"), "-lcudart",
                    "-Wl,-rpath," + os.path.join(cuda, "lib64")], check=True)
    return exe


@pytest.fixture(scope="session")
def gpu_api_test(lib):
    """tests/cpp/test_gpu_api.cpp built against the library (the C++ drop-in API with user
    potentials, NewtonsMethod on the GPU)."""
    import subprocess

    from symx_gb300.build import cuda_home

    libdir = os.path.join(ROOT, "symx_gb300", "_build")
    exe = os.path.join(libdir, "test_gpu_api")
    cuda = cuda_home()
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(cuda, "include"),
                    os.path.join(ROOT, "tests", "cpp", "test_gpu_api.cpp"), "-o", exe, "-L" + libdir, "-lsymxg",
                    "-Wl,-rpath," + libdir], check=True)
    return exe
