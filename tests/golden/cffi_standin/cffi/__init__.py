"""A stand-in for the part of cffi's ABI mode that the reference's gdtk/gas.py uses (test infrastructure).

The GPU machines have no cffi, and the drop-in test of the C ABI runs the reference's unmodified
gas.py there.  This module is put first on sys.path only when `import cffi` fails.  It offers:
  FFI.cdef(text)            C prototypes of int/double/char*/double* arguments and int/double results;
  FFI.dlopen(name)          a library whose functions are looked up on first use (as cffi's ABI mode
                            does, so prototypes of functions the library lacks are harmless);
  FFI.new("double[]", init | n), FFI.new("double *"), FFI.new("char[]", bytes | n);
  FFI.string(char_buffer)   the bytes up to the first NUL.
tests/test_abi_cpu.py checks it against the real cffi on the gas-model calls that need no GPU.
"""
import ctypes
import re

__version__ = "standin"

_SCALAR = {"int": ctypes.c_int, "double": ctypes.c_double, "char*": ctypes.c_char_p,
           "double*": ctypes.POINTER(ctypes.c_double), "int*": ctypes.POINTER(ctypes.c_int), "void": None}
_PROTO = re.compile(r"(\w+\s*\*?)\s*(\w+)\s*\(([^)]*)\)\s*;")


def _ctype(decl):
    """ctypes type of a C declaration such as 'int gm_i', 'char* name', 'double *x' or 'double'."""
    d = re.sub(r"\s*\*\s*", "* ", decl.strip())
    base = d[:d.rindex("*") + 1] if "*" in d else d.split()[0]
    key = base.replace(" ", "")
    if key not in _SCALAR:
        raise TypeError("cffi stand-in: unsupported C type %r" % decl)
    return _SCALAR[key]


class _Lib:
    def __init__(self, cdll, protos):
        self._cdll = cdll
        self._protos = protos

    def __getattr__(self, name):
        if name not in self._protos:
            raise AttributeError("function %s was not declared with cdef()" % name)
        restype, argtypes = self._protos[name]
        fn = getattr(self._cdll, name)   # AttributeError if the library lacks it, on first use only
        fn.restype = restype
        fn.argtypes = argtypes
        setattr(self, name, fn)
        return fn


class FFI:
    def __init__(self):
        self._protos = {}

    def cdef(self, text):
        text = re.sub(r"/\*.*?\*/|//[^\n]*", "", text, flags=re.S)
        for ret, name, args in _PROTO.findall(text):
            argv = [a for a in args.split(",") if a.strip() and a.strip() != "void"]
            self._protos[name] = (_ctype(ret), [_ctype(a) for a in argv])

    def dlopen(self, name):
        return _Lib(ctypes.CDLL(name), self._protos)

    def new(self, ctype, init=None):
        t = ctype.replace(" ", "")
        if t == "double*":
            return (ctypes.c_double * 1)()
        if t == "double[]":
            if isinstance(init, int):
                return (ctypes.c_double * init)()
            vals = list(init)
            return (ctypes.c_double * len(vals))(*vals)
        if t == "char[]":
            if isinstance(init, int):
                return ctypes.create_string_buffer(init)
            return ctypes.create_string_buffer(bytes(init), len(init))
        raise TypeError("cffi stand-in: unsupported ffi.new type %r" % ctype)

    @staticmethod
    def string(buf):
        return buf.value
