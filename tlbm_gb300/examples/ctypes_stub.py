"""Minimal ctypes binding of the C ABI (include/tlbm.h): create a handle from the input files
in the current directory, take 100 steps, write the dump files.  tlbm_gb300.TLBMPartition is
the full binding."""

import ctypes


def main():
    lib = ctypes.CDLL("tlbm_gb300/lib/libtlbm_gb300.so")
    lib.tlbm_create.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
                                ctypes.POINTER(ctypes.c_void_p)]
    lib.tlbm_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.tlbm_write_data.argtypes = [ctypes.c_void_p]
    h = ctypes.c_void_p()
    assert lib.tlbm_create(b".", 0, 1 << 20, ctypes.byref(h)) == 0
    for ts in range(100):
        lib.tlbm_step(h, ts % 2)
    lib.tlbm_write_data(h)


if __name__ == "__main__":
    main()
