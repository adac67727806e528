"""ctypes harness that calls a MEX gateway's ``mexFunction`` through the stub API.

TEST INFRASTRUCTURE ONLY.  It hosts (a) the reference's own gateways,
compiled unmodified into ``oracle/_ref/`` by ``oracle/Makefile``, and (b) the
drop-in gateway of this library, so both can be called with the argument lists
MATLAB would pass (``Helm3dmvp_mex.c:42-48``, ``Helm3dkaczswp_mex.c:43-50``).

Arrays are handed over as MATLAB would see them: column-major doubles with
separate real and imaginary parts (the pre-R2018a ``mxGetPr``/``mxGetPi`` API).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")


class MxArray(C.Structure):
    _fields_ = [
        ("m", C.c_size_t),
        ("n", C.c_size_t),
        ("pr", C.POINTER(C.c_double)),
        ("pi", C.POINTER(C.c_double)),
        ("owns", C.c_int),
    ]


class MexError(RuntimeError):
    """Raised when the gateway called mexErrMsgIdAndTxt; ``.ident`` holds the ID."""

    def __init__(self, ident: str):
        super().__init__(ident)
        self.ident = ident


class MexFunction:
    """One compiled MEX gateway (a shared object exporting mexFunction)."""

    def __init__(self, path: str):
        self.path = path
        self.lib = C.CDLL(path)
        self.lib.mexstub_call.restype = C.c_int
        self.lib.mexstub_call.argtypes = [
            C.c_int, C.POINTER(C.POINTER(MxArray)), C.c_int, C.POINTER(C.POINTER(MxArray)),
            C.c_char_p, C.c_size_t,
        ]
        self.lib.mexstub_destroy.argtypes = [C.POINTER(MxArray)]

    @staticmethod
    def _wrap(a, keep):
        """Build an mxArray view of a numpy value (kept alive through ``keep``)."""
        a = np.asarray(a)
        if a.ndim == 0:
            a = a.reshape(1, 1)
        elif a.ndim == 1:
            a = a.reshape(-1, 1)
        elif a.ndim > 2:
            a = a.reshape(a.shape[0], -1, order="F")
        mx = MxArray()
        mx.m, mx.n = a.shape[0], a.shape[1]
        re = np.asfortranarray(np.real(a), dtype=np.float64)
        keep.append(re)
        mx.pr = re.ctypes.data_as(C.POINTER(C.c_double))
        if np.iscomplexobj(a):
            im = np.asfortranarray(np.imag(a), dtype=np.float64)
            keep.append(im)
            mx.pi = im.ctypes.data_as(C.POINTER(C.c_double))
        else:
            mx.pi = C.POINTER(C.c_double)()
        mx.owns = 0
        keep.append(mx)
        return mx

    def __call__(self, *args):
        keep: list = []
        prhs_objs = [self._wrap(a, keep) for a in args]
        prhs = (C.POINTER(MxArray) * len(args))(*[C.pointer(m) for m in prhs_objs])
        plhs = (C.POINTER(MxArray) * 1)()
        err = C.create_string_buffer(256)
        rc = self.lib.mexstub_call(1, plhs, len(args), prhs, err, 256)
        if rc != 0:
            raise MexError(err.value.decode())
        out = plhs[0].contents
        m, n = out.m, out.n
        re = np.ctypeslib.as_array(out.pr, shape=(m * n,)).copy()
        if out.pi:
            im = np.ctypeslib.as_array(out.pi, shape=(m * n,)).copy()
            val = re + 1j * im
        else:
            val = re
        self.lib.mexstub_destroy(plhs[0])
        return val.reshape((m, n), order="F")


REF_NAMES = [
    "Helm3dmvp_forw_mex", "Helm3dmvp_forw_wnc_mex", "Helm3dmvp_forw_deriv_mex",
    "Helm3dmvp_adj_mex", "Helm3dmvp_adj_wnc_mex", "Helm3dmvp_adj_deriv_mex",
    "Helm3d_kacz_sweep_mex", "Helm3d_kacz_sweep_adj_mex", "Helm3d_kacz_sweep_wnc_mex",
    "Helm3d_kacz_sweep_wnc_fixed_mex",
]


def reference_available() -> bool:
    return all(os.path.exists(os.path.join(REF_DIR, n + ".so")) for n in REF_NAMES)


def load_reference(name: str) -> MexFunction:
    return MexFunction(os.path.join(REF_DIR, name + ".so"))
