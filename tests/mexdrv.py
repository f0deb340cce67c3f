"""Builds tests/mex_gateway_driver.cpp with the model and solver MEX
gateways against the project's MEX stand-in header into a shared library
loaded with ctypes (the gateways' mexFunction renamed gw_<name>)."""
import ctypes as C
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GATEWAYS = ("msot_model_mex", "rec_nn_with_L2_reg", "rec_nn_with_L1_eye_reg",
            "rec_nn_with_TV_reg")


def build(out_dir):
    from msot_gb300 import _build
    libdir = os.path.dirname(_build.LIB_PATH)
    inc = ["-I" + os.path.join(ROOT, "oracle", "mex_shim"), "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "mb-rec-msot_gb300", "mex")]
    objs = []
    for name in GATEWAYS:
        src = os.path.join(ROOT, "mb-rec-msot_gb300", "mex", name + ".cpp")
        obj = os.path.join(out_dir, name + ".o")
        subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-Wall", "-Werror", *inc,
                        f"-DmexFunction=gw_{name}", "-c", src, "-o", obj], check=True)
        objs.append(obj)
    so = os.path.join(out_dir, "libmexdrv.so")
    subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-shared", *inc,
                    os.path.join(ROOT, "tests", "mex_gateway_driver.cpp"), *objs, "-o", so,
                    "-L" + libdir, "-lmsotgpu", "-Wl,-rpath," + libdir], check=True)
    lib = C.CDLL(so)
    d, i, u, s, p = C.c_double, C.c_int, C.c_uint64, C.c_size_t, C.POINTER(C.c_double)
    lib.drv_create.argtypes = [i, i, i, i, d, p, p, i, i, p, d, i, C.POINTER(u), C.c_char_p, i]
    lib.drv_model.argtypes = [C.c_char_p, u, p, s, p, s, C.c_char_p, i]
    lib.drv_l2.argtypes = [u, p, s, i, d, C.c_char_p, d, C.c_char_p, p, s, p, C.c_char_p, i]
    lib.drv_l1_tv.argtypes = [i, u, p, s, i, d, p, s, p, C.c_char_p, i]
    lib.drv_error_case.argtypes = [i, C.c_char_p, i]
    return lib


def dptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))
