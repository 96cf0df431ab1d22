"""Per-call GPU form (libxingpu XinGpu* entry points, host pointers through the
C ABI) against the CPU oracle: bit-exact on seeded inputs, every size class,
every interpolation phase family, every transform type and size."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

BDS = (8, 10)


@pytest.fixture(scope="module", params=BDS)
def libs(request):
    from xin26x_gb300 import _lib
    bd = request.param
    g = _lib.load(bd)
    assert g.xin_gpu_init(0) == 0, g.xin_gpu_last_error()
    assert g.xin_gpu_bitdepth() == bd
    return g, O.oracle(bd), bd


def P(a, off=0):
    return O.ptr(a, off)


def _ok(g, what=""):
    assert g.xin_gpu_last_status() == 0, (what, g.xin_gpu_last_error())


SIZES = [(4, 4), (8, 8), (16, 16), (32, 32), (64, 64), (128, 128), (8, 4), (4, 16), (32, 8), (64, 16), (16, 128)]


def test_distortion_family(libs):
    g, o, bd = libs
    rng = np.random.default_rng(1)
    mx = (1 << bd) - 1
    for w, h in SIZES:
        stride = w + 7
        inp = rng.integers(0, mx + 1, size=(h, stride)).astype(o.pix)
        refs = [rng.integers(0, mx + 1, size=(h, stride + 3)).astype(o.pix) for _ in range(16)]
        rs = stride + 3
        a, b = np.zeros(8, np.uint32), np.zeros(8, np.uint32)
        g.XinGpuComputeSad(P(inp), stride, P(refs[0]), rs, w, h, P(a)); _ok(g)
        o.sad(P(inp), stride, P(refs[0]), rs, w, h, P(b))
        assert a[0] == b[0], (w, h)
        g.XinGpuComputeAvgSad(P(inp), stride, P(refs[0]), P(refs[1]), rs, w, h, P(a)); _ok(g)
        o.avg_sad(P(inp), stride, P(refs[0]), P(refs[1]), rs, w, h, P(b))
        assert a[0] == b[0]
        for wa in (-2, 3, 5, 10):
            g.XinGpuComputeWeightSad(P(inp), stride, P(refs[0]), P(refs[1]), rs, w, h, wa, 8 - wa, P(a)); _ok(g)
            o.weight_sad(P(inp), stride, P(refs[0]), P(refs[1]), rs, w, h, wa, 8 - wa, P(b))
            assert a[0] == b[0]
        ptrs = (C.c_void_p * 8)(*[refs[i].ctypes.data for i in range(8)])
        ptrsb = (C.c_void_p * 8)(*[refs[8 + i].ctypes.data for i in range(8)])
        g.XinGpuComputeSadx8(P(inp), stride, ptrs, rs, w, h, P(a)); _ok(g)
        o.sad_xn(P(inp), stride, ptrs, 8, rs, w, h, P(b))
        assert np.array_equal(a, b)
        g.XinGpuComputeSadx5(P(inp), stride, *[refs[i].ctypes.data for i in range(5)], rs, w, h, P(a)); _ok(g)
        o.sad_xn(P(inp), stride, ptrs, 5, rs, w, h, P(b))
        assert np.array_equal(a[:5], b[:5])
        g.XinGpuComputeSadx3(P(inp), stride, *[refs[i].ctypes.data for i in range(3)], rs, w, h, P(a)); _ok(g)
        o.sad_xn(P(inp), stride, ptrs, 3, rs, w, h, P(b))
        assert np.array_equal(a[:3], b[:3])
        g.XinGpuComputeAvgSadx8(P(inp), stride, ptrs, ptrsb, rs, w, h, P(a)); _ok(g)
        o.avg_sad_xn(P(inp), stride, ptrs, ptrsb, 8, rs, w, h, P(b))
        assert np.array_equal(a, b)
        g.XinGpuComputeVar(P(inp), stride, P(refs[2]), rs, w, h, P(a)); _ok(g)
        o.var(P(inp), stride, P(refs[2]), rs, w, h, P(b))
        assert a[0] == b[0]
        g.XinGpuComputeAvgVar(P(inp), stride, P(refs[2]), P(refs[3]), rs, w, h, P(a)); _ok(g)
        o.avg_var(P(inp), stride, P(refs[2]), P(refs[3]), rs, w, h, P(b))
        assert a[0] == b[0]
        g.XinGpuComputeSatd(P(inp), stride, P(refs[4]), rs, w, h, P(a)); _ok(g)
        o.satd(P(inp), stride, P(refs[4]), rs, w, h, P(b))
        assert a[0] == b[0], (w, h)
        g.XinGpuComputeAvgSatd(P(inp), stride, P(refs[4]), P(refs[5]), rs, w, h, P(a)); _ok(g)
        o.avg_satd(P(inp), stride, P(refs[4]), P(refs[5]), rs, w, h, P(b))
        assert a[0] == b[0]
        g.XinGpuComputeWeightSatd(P(inp), stride, P(refs[4]), P(refs[5]), rs, w, h, 3, 5, P(a)); _ok(g)
        o.weight_satd(P(inp), stride, P(refs[4]), P(refs[5]), rs, w, h, 3, 5, P(b))
        assert a[0] == b[0]
    blk = rng.integers(0, mx + 1, size=(8, 11)).astype(o.pix)
    g.XinGpuComputeHada8x8(P(blk), 11, P(a)); _ok(g)
    o.hada8x8(P(blk), 11, P(b))
    assert a[0] == b[0]


INTERP = [  # (gpu name, oracle name, taps, src s16, dst s16)
    ("InterpCopy", "interp_copy", 8, False, False), ("InterpCopyU8S16", "interp_copy_s16", 8, False, True),
    ("LumaInterpHor", "luma_hor", 8, False, False), ("LumaInterpVet", "luma_vet", 8, False, False),
    ("LumaInterpHorVet", "luma_hv", 8, False, False), ("LumaInterpHorU8S16", "luma_hor_s16", 8, False, True),
    ("LumaInterpVetU8S16", "luma_vet_s16", 8, False, True), ("LumaInterpHorVetU8S16", "luma_hv_s16", 8, False, True),
    ("LumaInterpVetS16U8", "luma_vet_s16_pix", 8, True, False), ("LumaInterpVetS16S16", "luma_vet_s16_s16", 8, True, True),
    ("ChromaInterpHor", "chroma_hor", 4, False, False), ("ChromaInterpVet", "chroma_vet", 4, False, False),
    ("ChromaInterpHorVet", "chroma_hv", 4, False, False), ("ChromaInterpHorU8S16", "chroma_hor_s16", 4, False, True),
    ("ChromaInterpVetU8S16", "chroma_vet_s16", 4, False, True), ("ChromaInterpHorVetU8S16", "chroma_hv_s16", 4, False, True),
    ("ChromaInterpVetS16U8", "chroma_vet_s16_pix", 4, True, False), ("ChromaInterpVetS16S16", "chroma_vet_s16_s16", 4, True, True),
]


@pytest.mark.parametrize("spec", INTERP, ids=[s[0] for s in INTERP])
def test_interpolation(libs, spec):
    g, o, bd = libs
    gname, oname, nt, s16, d16 = spec
    rng = np.random.default_rng(hash(gname) & 0xFFFF)
    mx = (1 << bd) - 1
    sizes = [(1, 1), (2, 4), (4, 4), (8, 8), (16, 16), (32, 32), (64, 64), (8, 2)]
    if nt == 8:
        sizes.append((128, 128))
    for w, h in sizes:
        m = 8
        if s16:
            src = rng.integers(-8192, 8192, size=(h + 2 * m, w + 2 * m + 5)).astype(np.int16)
        else:
            src = rng.integers(0, mx + 1, size=(h + 2 * m, w + 2 * m + 5)).astype(o.pix)
        sp = src.shape[1]
        off = m * sp + m
        dt = np.int16 if d16 else o.pix
        fracs = range(0, 256, 5) if nt == 8 else range(0, 1024, 19)
        for fi in ((0, 1, 2) if nt == 8 else (0,)):
            for frac in fracs:
                a = np.zeros((h, w + 3), dt)
                b = np.zeros((h, w + 3), dt)
                getattr(g, "XinGpu" + gname)(P(src, off), sp, P(a), w + 3, frac, w, h, fi)
                _ok(g, gname)
                getattr(o, oname)(P(src, off), sp, P(b), w + 3, frac, w, h, fi)
                assert np.array_equal(a, b), (gname, w, h, fi, frac)


def test_bilinear_interpolation(libs):
    """pfXinBiliInterp (DMVR bilinear prediction): the four variants at every
    tenth 1/16 phase and widths 1..128, h rows of w + 4 outputs, destination
    columns beyond w + 4 untouched."""
    g, o, bd = libs
    rng = np.random.default_rng(77)
    mx = (1 << bd) - 1
    for w, h in [(1, 1), (4, 4), (8, 16), (16, 8), (32, 32), (64, 64), (128, 128)]:
        src = rng.integers(0, mx + 1, size=(h + 4, w + 12)).astype(o.pix)
        sp = src.shape[1]
        for variant, name in enumerate(("Copy", "Hor", "Vet", "HorVet")):
            for frac in list(range(0, 256, 10)) + [255]:
                a = np.full((h, w + 9), 5, np.int16)
                b = np.full((h, w + 9), 5, np.int16)
                getattr(g, "XinGpuBiliInterp" + name)(P(src, sp + 1), sp, P(a), w + 9, frac, w, h)
                _ok(g, name)
                o.bili_interp(variant, P(src, sp + 1), sp, P(b), w + 9, frac, w, h)
                assert np.array_equal(a, b), (name, w, h, frac)


def test_interp_avg_weight(libs):
    g, o, bd = libs
    rng = np.random.default_rng(3)
    for w, h in [(2, 2), (4, 8), (16, 16), (64, 64), (128, 128)]:
        a = rng.integers(-8192, 8192, size=(h, w + 1)).astype(np.int16)
        b = rng.integers(-8192, 8192, size=(h, w + 2)).astype(np.int16)
        x = np.zeros((h, w), o.pix)
        y = np.zeros((h, w), o.pix)
        g.XinGpuInterpAvgS16U8(P(a), w + 1, P(b), w + 2, P(x), w, w, h); _ok(g)
        o.interp_avg(P(a), w + 1, P(b), w + 2, P(y), w, w, h)
        assert np.array_equal(x, y)
        for wa in (-2, 3, 4, 5, 10):
            g.XinGpuInterpWeightS16U8(P(a), w + 1, P(b), w + 2, P(x), w, w, h, wa, 8 - wa); _ok(g)
            o.interp_weight(P(a), w + 1, P(b), w + 2, P(y), w, w, h, wa, 8 - wa)
            assert np.array_equal(x, y)


ONE_D = [("Dct2", 0, (2, 4, 8, 16, 32, 64)), ("Dst7", 2, (4, 8, 16, 32)), ("Dct8", 1, (4, 8, 16, 32))]


def test_1d_transforms(libs):
    g, o, bd = libs
    rng = np.random.default_rng(5)
    lim = (1 << bd) - 1
    for name, ty, sizes in ONE_D:
        for n in sizes:
            lg = n.bit_length() - 1
            for line in (1, 4, 16, 64):
                x = rng.integers(-lim, lim + 1, size=(line, n + 2)).astype(o.coef)
                a = np.zeros((n, line + 1), o.coef)
                b = np.zeros((n, line + 1), o.coef)
                shift = lg + bd + 6 - 15
                getattr(g, f"XinGpuF{name}P{n}")(P(x), n + 2, P(a), line + 1, line, shift); _ok(g)
                o.fdct1d(ty, lg, P(x), n + 2, P(b), line + 1, line, shift)
                assert np.array_equal(a, b), ("F", name, n, line)
                c = np.clip(rng.laplace(0, 500, size=(n, line + 2)), -32768, 32767).astype(o.coef)
                for skip in {0, line // 2}:
                    for shift in (7, 20 - bd):
                        a = np.zeros((line, n + 1), o.coef)
                        b = np.zeros((line, n + 1), o.coef)
                        getattr(g, f"XinGpuI{name}P{n}")(P(c), line + 2, P(a), n + 1, line, skip, shift); _ok(g)
                        o.idct1d(ty, lg, P(c), line + 2, P(b), n + 1, line, skip, shift)
                        assert np.array_equal(a, b), ("I", name, n, line, skip)


def test_2d_dct2_skip_sub_add(libs):
    g, o, bd = libs
    rng = np.random.default_rng(7)
    lim = (1 << bd) - 1
    for w in (2, 4, 8, 16, 32, 64):
        for h in (2, 4, 8, 16, 32, 64):
            lw, lh = w.bit_length() - 1, h.bit_length() - 1
            x = rng.integers(-lim, lim + 1, size=(h, w + 1)).astype(o.coef)
            a = np.zeros((h, w + 2), o.coef)
            b = np.zeros((h, w + 2), o.coef)
            s1, s2 = lw + bd + 6 - 15, lh + 6
            g.XinGpuFDct2WxH(P(x), w + 1, P(a), w + 2, w, h, None, s1, s2); _ok(g)
            o.fdct2_wxh(P(x), w + 1, P(b), w + 2, w, h, s1, s2)
            assert np.array_equal(a, b), ("FDct2WxH", w, h)
            c = np.clip(rng.laplace(0, 300, size=(h, w + 1)), -32768, 32767).astype(o.coef)
            g.XinGpuIDct2WxH(P(c), w + 1, P(a), w + 2, w, h, None, 7, 20 - bd); _ok(g)
            o.idct2_wxh(P(c), w + 1, P(b), w + 2, w, h, 7, 20 - bd)
            assert np.array_equal(a, b), ("IDct2WxH", w, h)
            g.XinGpuFSkipWxH(P(x), w + 1, P(a), w + 2, w, h, None); _ok(g)
            o.fskip_wxh(P(x), w + 1, P(b), w + 2, w, h)
            assert np.array_equal(a, b)
            g.XinGpuISkipWxH(P(c), w + 1, P(a), w + 2, w, h); _ok(g)
            o.iskip_wxh(P(c), w + 1, P(b), w + 2, w, h)
            assert np.array_equal(a, b)
            inp = rng.integers(0, lim + 1, size=(h, w + 3)).astype(o.pix)
            prd = rng.integers(0, lim + 1, size=(h, w + 4)).astype(o.pix)
            g.XinGpuBlockSubForDct(P(inp), w + 3, P(prd), w + 4, P(a), w + 2, w, h); _ok(g)
            o.block_sub(P(inp), w + 3, P(prd), w + 4, P(b), w + 2, w, h)
            assert np.array_equal(a, b)
            r1 = np.zeros((h, w + 1), o.pix)
            r2 = np.zeros((h, w + 1), o.pix)
            g.XinGpuBlockAddForDct(P(c), w + 1, P(prd), w + 4, P(r1), w + 1, w, h); _ok(g)
            o.block_add(P(c), w + 1, P(prd), w + 4, P(r2), w + 1, w, h)
            assert np.array_equal(r1, r2)


def _scan_cg(wcg, hcg):
    out, x, y, n = [], 0, 0, 0
    while n < wcg * hcg:
        while y >= 0:
            if x < wcg and y < hcg:
                out.append((x, y, y * wcg + x))
                n += 1
            y -= 1
            x += 1
        y, x = x, 0
    return np.array(out, np.uint32)


def test_quant_and_prerdoq(libs):
    g, o, bd = libs
    rng = np.random.default_rng(9)
    for qp in range(0, 64, 5):
        for lgw, lgh in [(2, 2), (3, 3), (4, 4), (5, 5), (2, 5), (5, 3)]:
            w, h = 1 << lgw, 1 << lgh
            p = O.orc_qparams()
            o.quant_params(qp, lgw, lgh, qp % 2, qp % 3 == 0, qp % 4 == 0, p)
            t = np.clip(rng.laplace(0, 400, size=(h, w + 2)), -32768, 32767).astype(o.coef)
            outs = []
            for which in (0, 1):
                q = np.full((h, w + 2), 5, o.coef)
                r = np.full((h, w + 2), 5, o.coef)
                nz = np.zeros(1, np.uint64)
                f = g.XinGpuQuantInvQuant if which == 0 else o.quant_inv_quant
                f(P(q), P(t), P(r), w + 2, w, h, 4, 4, p.qmult, p.qadd, p.qshift, p.iqmult, p.iqadd, p.iqshift, P(nz))
                if which == 0:
                    _ok(g)
                outs.append((q, r, nz))
            for x, y in zip(*outs):
                assert np.array_equal(x, y), (qp, w, h)
    for lgw, lgh in [(2, 2), (3, 3), (4, 4), (5, 5), (3, 5)]:
        w, h = 1 << lgw, 1 << lgh
        scan = _scan_cg(w // 4, h // 4)
        for thr in (0, 8, 40, 200):
            t = np.clip(rng.laplace(0, 30, size=(h, w)), -32768, 32767).astype(o.coef)
            q0 = rng.integers(-3, 4, size=(h, w)).astype(o.coef)
            nblk = (w // 4) * (h // 4)
            nz0 = np.array([int(rng.integers(0, 1 << 62)) & ((1 << nblk) - 1)], np.uint64)
            outs = []
            for which in (0, 1):
                q, r, nz = q0.copy(), q0.copy() * 3, nz0.copy()
                f = g.XinGpuPreRdoq if which == 0 else o.pre_rdoq
                f(P(t), P(r), P(q), w, w, h, 4, 4, thr, P(scan), P(nz))
                if which == 0:
                    _ok(g)
                outs.append((q, r, nz))
            for x, y in zip(*outs):
                assert np.array_equal(x, y), (w, h, thr)


def _me_state(g_lib, inp, refp, pad, w, h, rng_range, mvp, lam, start, window):
    from xin26x_gb300 import _lib
    me = _lib.xin_gpu_me_struct()
    me.width, me.height = w, h
    me.input, me.inputStride = inp.ctypes.data, inp.shape[1]
    me.ref, me.refStride = refp.ctypes.data + (pad * refp.shape[1] + pad) * refp.itemsize, refp.shape[1]
    me.searchWidth = me.searchHeight = rng_range
    me.predMv.mvX, me.predMv.mvY = mvp
    me.bestMv.mvX, me.bestMv.mvY = start[:2]
    me.bestCost = start[2]
    me.bestSad = 12345
    me.minMv.mvX, me.minMv.mvY, me.maxMv.mvX, me.maxMv.mvY = window
    me.sadLambda = lam
    return me


def test_motion_search_drivers(libs):
    g, o, bd = libs
    rng = np.random.default_rng(11)
    mx = (1 << bd) - 1
    for w, h in [(8, 8), (16, 16), (32, 32), (64, 64), (16, 8), (8, 32)]:
        pad = 48
        base = rng.integers(0, mx + 1, size=(h + 2 * pad, w + 2 * pad)).astype(np.int32)
        refp = ((base + np.roll(base, 1, 0) + np.roll(base, 1, 1)) // 3).astype(o.pix)
        inp = np.ascontiguousarray(refp[pad + 5:pad + 5 + h, pad - 3:pad - 3 + w])
        for R, mvp, win in [(8, (0, 0), (-20, -20, 20, 20)), (12, (5, -7), (-9, -30, 4, 30)), (6, (-13, 2), (-40, -40, 40, 40))]:
            lam = int(rng.integers(0, 300))
            me = _me_state(g, inp, refp, pad, w, h, R, mvp, lam, (0, 0, 0xFFFFFFFF), win)
            g.XinGpuMotionEstFull(C.byref(me)); _ok(g, "MotionEstFull")
            io = O.orc_me_io(0, 0, 0xFFFFFFFF, 12345)
            o.me_full(P(inp), w, P(refp, pad * refp.shape[1] + pad), refp.shape[1], w, h, mvp[0], mvp[1], R, lam,
                      win[0], win[1], win[2], win[3], io)
            assert (me.bestMv.mvX, me.bestMv.mvY, me.bestCost, me.bestSad) == (io.best_mvx, io.best_mvy, io.best_cost, io.best_sad)
            g.XinGpuFullSubPelMe(C.byref(me)); _ok(g, "FullSubPelMe")
            o.full_subpel_me(P(inp), w, P(refp, pad * refp.shape[1] + pad), refp.shape[1], w, h, mvp[0], mvp[1], lam,
                             win[0], win[1], win[2], win[3], io)
            assert (me.bestMv.mvX, me.bestMv.mvY, me.bestCost) == (io.best_mvx, io.best_mvy, io.best_cost)
        # an incoming best that no candidate beats is kept
        me = _me_state(g, inp, refp, pad, w, h, 4, (0, 0), 10, (8, 4, 0), (-20, -20, 20, 20))
        g.XinGpuMotionEstFull(C.byref(me)); _ok(g)
        assert (me.bestMv.mvX, me.bestMv.mvY, me.bestCost, me.bestSad) == (8, 4, 0, 12345)


def test_motion_search_default_range(libs):
    """XinGpuMotionEstFull and XinGpuFullSubPelMe at the encoder's default range of
    +-64 (h26x_api/source/h26x_encoder_api.c:202) with a window wide enough that
    the clip does not shorten it, and one window that clips a side to 3."""
    g, o, bd = libs
    rng = np.random.default_rng(64)
    mx = (1 << bd) - 1
    R = 64
    for w, h in [(8, 8), (16, 16), (32, 32), (64, 64), (32, 8)]:
        pad = 96
        base = rng.integers(0, mx + 1, size=(h + 2 * pad, w + 2 * pad)).astype(np.int32)
        refp = ((base + np.roll(base, 1, 0) + np.roll(base, 2, 1)) // 3).astype(o.pix)
        inp = np.ascontiguousarray(refp[pad + 37:pad + 37 + h, pad - 51:pad - 51 + w])
        for mvp, win in [((0, 0), (-80, -80, 80, 80)), ((-9, 6), (-70, -3, 75, 80))]:
            lam = int(rng.integers(0, 300))
            me = _me_state(g, inp, refp, pad, w, h, R, mvp, lam, (0, 0, 0xFFFFFFFF), win)
            g.XinGpuMotionEstFull(C.byref(me)); _ok(g, "MotionEstFull")
            io = O.orc_me_io(0, 0, 0xFFFFFFFF, 12345)
            o.me_full(P(inp), w, P(refp, pad * refp.shape[1] + pad), refp.shape[1], w, h, mvp[0], mvp[1], R, lam,
                      win[0], win[1], win[2], win[3], io)
            assert (me.bestMv.mvX, me.bestMv.mvY, me.bestCost, me.bestSad) == \
                (io.best_mvx, io.best_mvy, io.best_cost, io.best_sad), (w, h, mvp)
            g.XinGpuFullSubPelMe(C.byref(me)); _ok(g, "FullSubPelMe")
            o.full_subpel_me(P(inp), w, P(refp, pad * refp.shape[1] + pad), refp.shape[1], w, h, mvp[0], mvp[1], lam,
                             win[0], win[1], win[2], win[3], io)
            assert (me.bestMv.mvX, me.bestMv.mvY, me.bestCost) == (io.best_mvx, io.best_mvy, io.best_cost)


def _down(o, plane, levels=2):
    out, src = [], np.ascontiguousarray(plane)
    for _ in range(levels):
        h, w = src.shape[0] // 2, src.shape[1] // 2
        d = np.zeros((h, w), src.dtype)
        o.downscale2x2(P(src), src.shape[1], 0, 0, P(d), w, w, h)
        out.append(d)
        src = d
    return out


def test_downscale2x2(libs):
    """XinGpuDownscale2x2 against the oracle's restatement, odd output sizes and
    strides; the row flags (never set by the reference's callers) are refused."""
    g, o, bd = libs
    rng = np.random.default_rng(22)
    mx = (1 << bd) - 1
    for ow, oh in [(1, 1), (7, 5), (64, 32), (133, 71), (960, 540)]:
        src = rng.integers(0, mx + 1, size=(2 * oh + 3, 2 * ow + 5)).astype(o.pix)
        a = np.full((oh, ow + 2), 7, o.pix)
        b = a.copy()
        g.XinGpuDownscale2x2(P(src), src.shape[1], 0, 0, P(a), ow + 2, ow, oh); _ok(g)
        o.downscale2x2(P(src), src.shape[1], 0, 0, P(b), ow + 2, ow, oh)
        assert np.array_equal(a, b), (ow, oh)
    g.XinGpuDownscale2x2(P(src), src.shape[1], 1, 0, P(a), ow + 2, ow, oh)
    assert g.xin_gpu_last_status() == -2


def test_motion_search_hier_level(libs):
    """XinGpuMotionSearchHier (one level): every MV of the window, SAD, strict '<'
    in raster order; an empty window leaves the output unchanged."""
    from xin26x_gb300 import _lib
    g, o, bd = libs
    rng = np.random.default_rng(23)
    mx = (1 << bd) - 1
    pad = 40
    for w, h in [(2, 2), (4, 4), (8, 8), (16, 16), (4, 8), (32, 16)]:
        base = rng.integers(0, mx + 1, size=(h + 2 * pad, w + 2 * pad)).astype(np.int32)
        refp = ((base + np.roll(base, 1, 1)) // 2).astype(o.pix)
        inp = np.ascontiguousarray(refp[pad + 3:pad + 3 + h, pad - 6:pad - 6 + w])
        for win in [(-16, 16, -16, 16), (-3, 9, 0, 0), (5, 30, -30, -2), (4, 3, 0, 0)]:
            mv = _lib.xin_gpu_mv()
            mv.mvX, mv.mvY = 77, -77
            g.XinGpuMotionSearchHier(P(inp), w, P(refp, pad * refp.shape[1] + pad), refp.shape[1], win[0], win[1],
                                     win[2], win[3], w, h, C.byref(mv)); _ok(g)
            bx, by = C.c_int32(77), C.c_int32(-77)
            o.hier_search(P(inp), w, P(refp, pad * refp.shape[1] + pad), refp.shape[1], win[0], win[1], win[2], win[3],
                          w, h, C.byref(bx), C.byref(by))
            assert (mv.mvX, mv.mvY) == (bx.value, by.value), (w, h, win)


def test_motion_est_hier_driver(libs):
    """XinGpuMotionEstHier on the reference's ME state against the oracle's
    restatement (orc_me_hier): levels downscaled from the padded reference and
    the current picture, candidate lists, predictors, windows that clip, ranges
    up to the encoder's default +-64."""
    from xin26x_gb300 import _lib
    g, o, bd = libs
    rng = np.random.default_rng(24)
    mx = (1 << bd) - 1
    pad = 96
    H, W = 128, 192
    base = rng.integers(0, mx + 1, size=(H + 2 * pad, W + 2 * pad)).astype(np.int32)
    refp = ((base + np.roll(base, 1, 0) + np.roll(base, 1, 1) + np.roll(base, 3, 1)) // 4).astype(o.pix)
    cur = np.ascontiguousarray(np.roll(refp, (5, -13), (0, 1))[pad:pad + H, pad:pad + W])
    ref_lo, cur_lo = _down(o, refp), _down(o, cur)
    for (w, h, px, py) in [(8, 8, 16, 8), (16, 16, 64, 32), (32, 32, 96, 64), (64, 64, 64, 64), (16, 8, 8, 40)]:
        for R, mvp, win, cands in [(16, (0, 0), (-40, -40, 40, 40), [(0, 0)]),
                                   (64, (-20, 12), (-80, -70, 75, 60), [(0, 0), (-20, 12), (52, -9)]),
                                   (24, (8, 8), (-10, -3, 6, 90), [(0, 0), (8, 8), (400, -400)])]:
            lam = int(rng.integers(0, 300))
            me = _lib.xin_gpu_me_struct()
            me.width, me.height = w, h
            me.input, me.inputStride = P(cur, py * W + px), W
            me.input1, me.input1Stride = P(cur_lo[0], (py // 2) * cur_lo[0].shape[1] + px // 2), cur_lo[0].shape[1]
            me.input2, me.input2Stride = P(cur_lo[1], (py // 4) * cur_lo[1].shape[1] + px // 4), cur_lo[1].shape[1]
            rs = [refp.shape[1], ref_lo[0].shape[1], ref_lo[1].shape[1]]
            me.ref, me.refStride = P(refp, (pad + py) * rs[0] + pad + px), rs[0]
            me.ref1, me.ref1Stride = P(ref_lo[0], (pad // 2 + py // 2) * rs[1] + pad // 2 + px // 2), rs[1]
            me.ref2, me.ref2Stride = P(ref_lo[1], (pad // 4 + py // 4) * rs[2] + pad // 4 + px // 4), rs[2]
            me.searchWidth = me.searchHeight = R
            me.predMv.mvX, me.predMv.mvY = mvp
            me.bestMv.mvX, me.bestMv.mvY = 0, 0
            me.bestCost, me.bestSad = 0xFFFFFFFF, 0
            me.minMv.mvX, me.minMv.mvY, me.maxMv.mvX, me.maxMv.mvY = win
            me.sadLambda = lam
            me.candNum = len(cands)
            for i, (cx, cy) in enumerate(cands):
                me.meCand[i].mvX, me.meCand[i].mvY = cx, cy
            g.XinGpuMotionEstHier(C.byref(me)); _ok(g, "MotionEstHier")
            hin = O.orc_hier_in()
            for l, (ip_, ist, rp_, rst) in enumerate([(me.input, W, me.ref, rs[0]), (me.input1, me.input1Stride, me.ref1, rs[1]),
                                                      (me.input2, me.input2Stride, me.ref2, rs[2])]):
                hin.in_[l], hin.in_stride[l], hin.ref[l], hin.ref_stride[l] = ip_, ist, rp_, rst
            ca = np.array(cands, np.int32).reshape(-1)
            hin.cand, hin.ncand = ca.ctypes.data, len(cands)
            io = O.orc_me_io(0, 0, 0xFFFFFFFF, 0)
            o.me_hier(C.byref(hin), w, h, mvp[0], mvp[1], R, R, lam, win[0], win[1], win[2], win[3], io)
            assert (me.bestMv.mvX, me.bestMv.mvY, me.bestCost, me.bestSad) == \
                (io.best_mvx, io.best_mvy, io.best_cost, io.best_sad), (w, h, R, mvp)


def test_dmvr_helpers(libs):
    """pfXinComputeSadS16 (row-subsampled int16 SAD) and pfXinCopyAndPad / Uv
    against the oracle (itself pinned to h266_copy_and_pad.c compiled in place)."""
    g, o, bd = libs
    rng = np.random.default_rng(540)
    for w, h in [(8, 8), (16, 16), (16, 8), (8, 32), (64, 64), (128, 16)]:
        a = rng.integers(-9000, 9000, size=(h, w + 5)).astype(np.int16)
        b = rng.integers(-9000, 9000, size=(h, w + 2)).astype(np.int16)
        for sub in (0, 1, 2):
            x, y = np.zeros(1, np.uint32), np.zeros(1, np.uint32)
            g.XinGpuComputeSadS16(P(a), w + 5, P(b), w + 2, w, h, sub, P(x)); _ok(g)
            o.sad_s16(P(a), w + 5, P(b), w + 2, w, h, sub, P(y))
            assert x[0] == y[0], (w, h, sub)
    src = rng.integers(0, (1 << bd), size=(80, 96)).astype(o.pix)
    srcv = rng.integers(0, (1 << bd), size=(80, 96)).astype(o.pix)
    for w, h in [(4, 4), (8, 8), (16, 16), (8, 16), (16, 4)]:
        bufs = [np.full((32, 32), 5, o.pix) for _ in range(4)]
        off = 8 * 32 + 8
        g.XinGpuCopyAndPad(P(src, 20 * 96 + 30), 96, P(bufs[0], off), 32, w, h); _ok(g)
        o.copy_and_pad(P(src, 20 * 96 + 30), 96, P(bufs[1], off), 32, w, h)
        assert np.array_equal(bufs[0], bufs[1]), (w, h)
        g.XinGpuCopyAndPadUv(P(src, 20 * 96 + 30), P(srcv, 20 * 96 + 30), 96, P(bufs[0], off), P(bufs[2], off), 32, w, h)
        _ok(g)
        o.copy_and_pad_uv(P(src, 20 * 96 + 30), P(srcv, 20 * 96 + 30), 96, P(bufs[1], off), P(bufs[3], off), 32, w, h)
        assert np.array_equal(bufs[0], bufs[1]) and np.array_equal(bufs[2], bufs[3]), (w, h)


def test_dmvr_luma(libs):
    """XinGpuLumaMotionCompDmvr against the oracle's restatement of
    Xin266LumaMotionCompDmvr / Xin266DeriveMvFromDmvr (pinned to the compiled
    reference): sub-block refinements and the refined bi-prediction, every
    block size 8..128, shifted reference pairs, flat blocks, clipped windows and
    the alternative half-pel filter."""
    g, o, bd = libs
    rng = np.random.default_rng(975 + bd)
    pad = 80
    H, W = 160, 224
    base = rng.integers(0, 1 << bd, size=(H + 2 * pad, W + 2 * pad)).astype(np.int32)
    sm = ((base + np.roll(base, 1, 0) + np.roll(base, 1, 1) + np.roll(base, (1, 1), (0, 1))) // 4).astype(o.pix)
    rs = sm.shape[1]
    sizes = [(8, 16), (16, 8), (16, 16), (32, 16), (32, 32), (64, 64), (128, 128), (16, 64), (64, 8), (8, 8)]
    moved = 0
    for trial in range(160):
        w, h = sizes[trial % len(sizes)]
        sx, sy = int(rng.integers(-3, 4)), int(rng.integers(-3, 4))
        ref1 = np.ascontiguousarray(np.roll(sm, (sy, sx), (0, 1)))
        if trial % 9 == 4:
            ref1 = np.full_like(sm, 77)
        cx = int(rng.integers(0, (W - w) // 8 + 1)) * 8
        cy = int(rng.integers(0, (H - h) // 8 + 1)) * 8
        mv = np.array(rng.integers(-120, 121, 4), np.int32)
        win = (-cx - 72, -cy - 72, W + 72 - w - cx, H + 72 - h - cy) if trial % 5 else (-3, -2, 4, 3)
        n = (w // min(w, 16)) * (h // min(h, 16))
        outs = []
        for which in (0, 1):
            mvd = np.zeros(2 * n, np.int16)
            pred = np.zeros((h, w + 3), o.pix)
            args = (P(sm, pad * rs + pad), P(ref1, pad * rs + pad), rs, cx, cy, *win, w, h, P(mv), int(trial % 4 == 1))
            if which == 0:
                g.XinGpuLumaMotionCompDmvr(*args, P(pred), w + 3, P(mvd)); _ok(g, "dmvr")
            else:
                o.dmvr_luma(*args, P(mvd), P(pred), w + 3)
            outs.append((mvd, pred))
        assert np.array_equal(outs[0][0], outs[1][0]), ("mvd", trial, w, h, outs[0][0], outs[1][0])
        assert np.array_equal(outs[0][1], outs[1][1]), ("pred", trial, w, h)
        moved += int(np.any(outs[1][0] != 0))
    assert moved > 30


def test_fast_subpel_me_var(libs):
    """XinGpuFastSubPelMeVar against the oracle's restatement of Xin266FastSubPelMeVar
    (pinned to the compiled reference on the reference's buffer layout), with and
    without half-pel AMVR, starts inside and outside the window; and
    XinGpuInterpoHalfPel's four planes in the ME state's layout."""
    from xin26x_gb300 import _lib
    g, o, bd = libs
    rng = np.random.default_rng(2007 + bd)
    mx = (1 << bd) - 1
    pad = 48
    for w, h in [(8, 8), (16, 16), (32, 32), (64, 64), (128, 128), (16, 8), (8, 32)]:
        base = rng.integers(0, mx + 1, size=(h + 2 * pad, w + 2 * pad)).astype(np.int32)
        refp = ((base + np.roll(base, 1, 0) + np.roll(base, 1, 1)) // 3).astype(o.pix)
        inp = np.ascontiguousarray(refp[pad + 2:pad + 2 + h, pad - 1:pad - 1 + w] // 2 + 3).astype(o.pix)
        rs = refp.shape[1]
        for trial in range(10):
            mv = (int(rng.integers(-6, 7)) * 4, int(rng.integers(-6, 7)) * 4)
            mvp = (int(rng.integers(-20, 21)), int(rng.integers(-20, 21)))
            lam = int(rng.integers(0, 1 << 24))
            imv = 3 if trial % 3 == 2 else 0
            win = (-8, -8, 8, 8) if trial % 4 else (mv[0] // 4 + 1, -8, 8, 8)
            me = _lib.xin_gpu_me_struct()
            me.width, me.height = w, h
            me.input, me.inputStride = P(inp), w
            me.ref, me.refStride = P(refp, pad * rs + pad), rs
            me.predMv.mvX, me.predMv.mvY = mvp
            me.bestMv.mvX, me.bestMv.mvY = mv
            me.bestPos = 77
            me.minMv.mvX, me.minMv.mvY, me.maxMv.mvX, me.maxMv.mvY = win
            me.sseLambda, me.iMvMode = lam, imv
            g.XinGpuFastSubPelMeVar(C.byref(me), 0, 0); _ok(g, "FastSubPelMeVar")
            io = np.array([mv[0], mv[1], 77], np.int32)
            o.fast_subpel_me_var(P(inp), w, P(refp, pad * rs + pad), rs, w, h, mvp[0], mvp[1], lam, imv, *win, P(io))
            assert (me.bestMv.mvX, me.bestMv.mvY, me.bestPos) == tuple(int(v) for v in io), (w, h, trial)
        for alt in (0, 1):
            S = 200
            a = [np.full(S * S, 9, o.pix) for _ in range(4)]
            b = [np.full(S * S, 9, o.pix) for _ in range(4)]
            g.XinGpuInterpoHalfPel(P(refp, pad * rs + pad), rs, w, h, *[P(x) for x in a], S, alt); _ok(g)
            o.interpo_half_pel(P(refp, pad * rs + pad), rs, w, h, *[P(x) for x in b], S, alt)
            for k in range(4):
                assert np.array_equal(a[k], b[k]), (w, h, alt, k)


def test_invalid_arguments_report_errors(libs):
    g, o, bd = libs
    a = np.zeros(64, o.pix)
    out = np.array([7], np.uint32)
    g.XinGpuComputeSad(P(a), 8, P(a), 8, 0, 8, P(out))
    assert g.xin_gpu_last_status() == -2 and out[0] == 7
    g.XinGpuComputeSatd(P(a), 8, P(a), 8, 6, 6, P(out))
    assert g.xin_gpu_last_status() == -2
    g.XinGpuComputeSad(P(a), 8, P(a), 8, 8, 8, P(out))
    assert g.xin_gpu_last_status() == 0 and out[0] == 0
