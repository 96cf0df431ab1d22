"""Host-side parts of the serving layer that need no GPU: the device-footprint
arithmetic that admission uses, and its argument checks."""
import ctypes as C

import pytest

from xin26x_gb300 import _lib


def _fp(lib, w, h, ctu=64, r=64, mask=120, out=0, dio=0):
    cfg = _lib.xin_gpu_stream_cfg(w, h, ctu, r, mask, out, 1, dio)
    d, hb = C.c_uint64(), C.c_uint64()
    st = lib.xin_gpu_stream_footprint(C.byref(cfg), C.byref(d), C.byref(hb))
    return st, d.value, hb.value


@pytest.mark.parametrize("bd", (8, 10))
def test_footprint_arithmetic(bd):
    lib = _lib.load(bd)
    es = 1 if bd == 8 else 2          # pixel bytes
    cs = 2 if bd == 8 else 4          # coefficient bytes
    st, d, h = _fp(lib, 1920, 1080)
    assert st == 0
    # margin max(ctu + 16, R + 72) rounded to 32 -> 160; pitch rounded to 128 -> 2304 x 1400
    ysz, csz = 2304 * 1400 * es, 1152 * 700 * es
    ncus = 30 * 16 + 60 * 33 + 120 * 67 + 240 * 135
    lq = 1920 * 1080
    # two slots + quarter-pel planes, and two picture sets (search keys, CU records,
    # coefficient and reconstruction planes of four levels, a parameter block each)
    want = 2 * (ysz + 2 * csz) + 32 * ysz + 2 * (8 * ncus + 64 * ncus + lq * 3 // 2 * 4 * (cs + es))
    assert want < d < want + 8192
    assert h >= 2 * (64 * ncus + lq * 3 // 2 * es)
    # a wider search needs a wider margin; dropping levels drops their outputs
    assert _fp(lib, 1920, 1080, r=256)[1] > d
    assert _fp(lib, 1920, 1080, mask=64)[1] < d
    assert _fp(lib, 1920, 1080, dio=1)[2] < h
    for bad in ((1921, 1080), (8, 8)):
        assert _fp(lib, *bad)[0] == -2
    assert _fp(lib, 1920, 1080, ctu=32)[0] == -2
    assert _fp(lib, 1920, 1080, r=300)[0] == -2
    assert lib.xin_gpu_stream_footprint(None, None, None) == -2


def test_footprint_8bit_input_into_10bit_build():
    """input_bitdepth 8 in the 10-bit library: 8-bit device staging per picture set
    and 1-byte host staging; the 8-bit library accepts 0 and 8 only."""
    lib10, lib8 = _lib.load(10), _lib.load(8)

    def fp(lib, inb, dio=0):
        cfg = _lib.xin_gpu_stream_cfg(1920, 1080, 64, 64, 120, 0, 1, dio, inb)
        d, hb = C.c_uint64(), C.c_uint64()
        return lib.xin_gpu_stream_footprint(C.byref(cfg), C.byref(d), C.byref(hb)), d.value, hb.value

    st, d0, h0 = fp(lib10, 0)
    st8, d8, h8 = fp(lib10, 8)
    assert st == 0 and st8 == 0
    lq = 1920 * 1080
    assert d8 - d0 == 2 * lq * 3 // 2
    assert h0 - h8 == 2 * lq * 3 // 2
    assert fp(lib10, 8, dio=1)[1] == fp(lib10, 0, dio=1)[1]
    assert fp(lib10, 10)[0] == 0 and fp(lib10, 9)[0] == -2 and fp(lib10, 12)[0] == -2
    assert fp(lib8, 8)[0] == 0 and fp(lib8, 0)[0] == 0 and fp(lib8, 10)[0] == -2


@pytest.mark.parametrize("bd", (8, 10))
def test_footprint_two_references(bd):
    """refs 2: a third picture slot with its quarter-pel planes, list 1's search keys
    and a bi record per CU in each picture set (pinned host copies too); refused
    with the 128 x 128 level or more than two references."""
    lib = _lib.load(bd)
    es = 1 if bd == 8 else 2

    def fp(refs, tu=0, mask=120, ctu=64, sm=0):
        cfg = _lib.xin_gpu_stream_cfg(1920, 1080, ctu, 64, mask, 0, 1, 0, 0, sm, tu, refs)
        d, hb = C.c_uint64(), C.c_uint64()
        return lib.xin_gpu_stream_footprint(C.byref(cfg), C.byref(d), C.byref(hb)), d.value, hb.value

    st1, d1, h1 = fp(1)
    st2, d2, h2 = fp(2)
    assert st1 == 0 and st2 == 0 and fp(0)[1:] == (d1, h1)
    ysz, csz = 2304 * 1400 * es, 1152 * 700 * es
    ncus = 30 * 16 + 60 * 33 + 120 * 67 + 240 * 135
    assert d2 - d1 == (ysz + 2 * csz) + 16 * ysz + 2 * 8 * ncus + 2 * 40 * ncus    # keys per set; xin_gpu_cu_bi: 40 bytes
    assert h2 - h1 == 2 * 40 * ncus
    assert fp(3)[0] == -2 and fp(-1)[0] == -2 and fp(2, tu=1)[0] == 0
    assert fp(2, mask=248, ctu=128, sm=1)[0] == -2 and fp(1, mask=248, ctu=128, sm=1)[0] == 0
