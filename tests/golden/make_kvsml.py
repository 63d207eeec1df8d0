"""Generate the KVSML and AVS-field ingest fixtures from the reference.

Small structured volumes are written by the reference's own writer
(StructuredVolumeObject::write: inline ASCII, external ASCII, external
binary) into tests/golden/kvsml/, plus hand-made variants of those files
(big-endian binary data, only one of min_value / max_value, no coordinate
attributes, inline values separated by commas, tabs and newlines).  Every
file is then read back by the reference reader (StructuredVolumeObject::read)
and what it produced -- values, type, resolution, min/max, coordinates -- is
stored in tests/golden/kvsml/expected.npz with the case list in
tests/golden/kvsml/cases.json.  AVS field files (.fld: header lines, "\f\f",
raw values) are written here and read by the reference kvs::AVSField with the
StructuredVolumeImporter rules (kvsref_read_avs in oracle/ref_driver.cpp).

    python tests/golden/make_kvsml.py
"""
import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "kvsml")
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref  # noqa: E402


class RefVolume(C.Structure):
    _fields_ = [("success", C.c_int), ("dtype", C.c_int), ("nx", C.c_uint), ("ny", C.c_uint), ("nz", C.c_uint),
                ("veclen", C.c_uint), ("grid_type", C.c_int), ("vmin", C.c_double), ("vmax", C.c_double),
                ("min_obj", C.c_float * 3), ("max_obj", C.c_float * 3), ("min_ext", C.c_float * 3),
                ("max_ext", C.c_float * 3), ("nbytes", C.c_ulonglong), ("values", C.POINTER(C.c_ubyte))]


def lib():
    L = ref.lib()
    L.kvsref_write_kvsml.restype = C.c_int
    L.kvsref_write_kvsml.argtypes = [C.c_int, C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_char_p, C.c_int, C.c_int,
                                     C.c_int, C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_void_p]
    L.kvsref_read_kvsml.restype = C.c_int
    L.kvsref_read_kvsml.argtypes = [C.c_char_p, C.POINTER(RefVolume)]
    L.kvsref_free_volume.argtypes = [C.POINTER(RefVolume)]
    L.kvsref_read_avs.restype = C.c_int
    L.kvsref_read_avs.argtypes = [C.c_char_p, C.POINTER(RefVolume)]
    return L


def write_avs(name, v, data, ext=None, extra=""):
    """An AVS field file as the format defines it: '# AVS' line, key = value
    lines, two form feeds, the raw values (little-endian)."""
    nz, ny, nx = v.shape
    head = ["# AVS field file", "# written for the ingest fixtures", "#", "nspace = 3", "veclen = 1", "ndim   = 3",
            f"dim1   = {nx}", f"dim2   = {ny}", f"dim3   = {nz}", f"data   = {data}", "field  = uniform"]
    if ext:
        head += ["min_ext = %r %r %r" % tuple(ext[0]), "max_ext = %r %r %r" % tuple(ext[1])]
    head += ["label  = value"] + ([extra] if extra else [])
    with open(os.path.join(OUT, name + ".fld"), "wb") as f:
        f.write(("\n".join(head) + "\n").encode())
        f.write(b"\f\f")
        f.write(np.ascontiguousarray(v).astype(v.dtype.newbyteorder("<")).tobytes())


def write(name, v, ascii, external, minmax=None, obj=None):
    p = os.path.join(OUT, name + ".kvsml")
    mn = np.ascontiguousarray(obj[0], np.float32) if obj else None
    mx = np.ascontiguousarray(obj[1], np.float32) if obj else None
    v = np.ascontiguousarray(v)
    nz, ny, nx = v.shape
    rc = lib().kvsref_write_kvsml(ref.dtype_code(v.dtype), v.ctypes.data, nx, ny, nz, p.encode(), int(ascii),
                                  int(external), 1 if minmax else 0, minmax[0] if minmax else 0.0,
                                  minmax[1] if minmax else 0.0, 1 if obj else 0,
                                  mn.ctypes.data if obj else None, mx.ctypes.data if obj else None)
    assert rc == 0, name
    return p


def edit(src, dst, fn):
    text = open(os.path.join(OUT, src + ".kvsml")).read()
    open(os.path.join(OUT, dst + ".kvsml"), "w").write(fn(text))


def main():
    if not ref.available():
        ref.build()
    os.makedirs(OUT, exist_ok=True)
    for f in os.listdir(OUT):
        os.remove(os.path.join(OUT, f))
    rng = np.random.default_rng(99)
    shape = (5, 6, 7)
    f32 = rng.random(shape).astype(np.float32) * 10 - 3
    u8 = rng.integers(0, 256, shape).astype(np.uint8)
    i16 = rng.integers(-3000, 3000, shape).astype(np.int16)
    u16 = rng.integers(0, 65536, shape).astype(np.uint16)
    i8 = rng.integers(-128, 128, shape).astype(np.int8)
    f64 = rng.standard_normal(shape)
    i32 = rng.integers(-2 ** 31, 2 ** 31 - 1, shape).astype(np.int32)
    u32 = rng.integers(0, 2 ** 32 - 1, shape).astype(np.uint32)
    for name, v in (("f32", f32), ("u8", u8)):
        write(f"{name}_ascii", v, 1, 0)
        write(f"{name}_extascii", v, 1, 1)
        write(f"{name}_binary", v, 0, 1)
    write("i16_binary", i16, 0, 1)
    write("i16_ascii", i16, 1, 0)
    write("u16_binary", u16, 0, 1)
    write("i8_ascii", i8, 1, 0)
    write("f64_binary", f64, 0, 1)
    write("i32_binary", i32, 0, 1)
    write("u32_extascii", u32, 1, 1)
    write("f32_coords", f32, 0, 1, minmax=(-5.0, 9.5), obj=([1.5, -2.0, 0.25], [8.0, 3.0, 4.75]))
    # big-endian copy of the binary float data
    raw = np.fromfile(os.path.join(OUT, "f32_binary_value.dat"), "<f4")
    raw.astype(">f4").tofile(os.path.join(OUT, "f32_big_value.dat"))
    edit("f32_binary", "f32_big", lambda t: t.replace('file="f32_binary_value.dat" endian="little"',
                                                     'file="f32_big_value.dat" endian="big"'))
    # min_value only (the max comes from the scan); no coordinate attributes
    edit("f32_binary", "f32_minonly",
         lambda t: __import__("re").sub(r' max_value="[^"]*"', "", t).replace(' min_value="', ' min_value="-1.25" x="'))
    edit("f32_binary", "f32_nocoord",
         lambda t: __import__("re").sub(r' (external|object)_coord="[^"]*"', "", t))
    # inline values separated by commas, tabs and newlines
    vals = ",".join(f"{x:.9g}" for x in f32.ravel()[:100]) + "\n\t" + " ,".join(f"{x:.9g}" for x in f32.ravel()[100:])
    text = open(os.path.join(OUT, "f32_ascii.kvsml")).read()
    start = text.index('<DataArray type="float">') + len('<DataArray type="float">')
    end = text.index("</DataArray>")
    open(os.path.join(OUT, "f32_commas.kvsml"), "w").write(text[:start] + vals + "\n" + text[end:])
    # AVS fields
    write_avs("avs_f32", f32, "float", ext=([0.5, -1.0, 2.0], [7.5, 4.0, 6.0]))
    write_avs("avs_u8", u8, "byte")
    write_avs("avs_i16", i16, "short", extra="# comment after the keys")
    write_avs("avs_i32", i32, "integer")
    write_avs("avs_f64", f64, "double", extra="unknown_key = 12")
    # what the reference reader makes of every file
    arrays, cases = {}, []
    for fn in sorted(f for f in os.listdir(OUT) if f.endswith(".kvsml") or f.endswith(".fld")):
        name = fn.rsplit(".", 1)[0]
        r = RefVolume()
        read = lib().kvsref_read_avs if fn.endswith(".fld") else lib().kvsref_read_kvsml
        assert read(os.path.join(OUT, fn).encode(), C.byref(r)) == 0, fn
        dt = np.dtype(ref.DTYPES[r.dtype])
        vals = np.ctypeslib.as_array(r.values, shape=(r.nbytes,)).copy().view(dt).reshape(r.nz, r.ny, r.nx)
        arrays[name] = vals
        cases.append(dict(name=name, file=fn, dtype=dt.name, resolution=[r.nx, r.ny, r.nz], veclen=r.veclen,
                          vmin=r.vmin, vmax=r.vmax, min_obj=list(r.min_obj), max_obj=list(r.max_obj),
                          min_ext=list(r.min_ext), max_ext=list(r.max_ext)))
        lib().kvsref_free_volume(C.byref(r))
    np.savez_compressed(os.path.join(OUT, "expected.npz"), **arrays)
    with open(os.path.join(OUT, "cases.json"), "w") as f:
        json.dump(cases, f, indent=0)
    print(f"{len(cases)} kvsml/avs cases, {sum(os.path.getsize(os.path.join(OUT, x)) for x in os.listdir(OUT))} bytes")


if __name__ == "__main__":
    main()
