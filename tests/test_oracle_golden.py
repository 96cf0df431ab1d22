"""Replay the golden fixtures (outputs of the reference's own open C, made by
tests/golden/make_golden.py) through the oracle.  Runs anywhere: it needs
neither the reference tree nor a GPU."""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("bd", (8, 10))
def test_golden(bd):
    g = np.load(os.path.join(GOLD, f"ref_golden_{bd}bit.npz"))
    o = O.oracle(bd)
    src, s16 = g["interp_src"], g["interp_s16"]
    for key in g.files:
        if not key.startswith("interp_") or key in ("interp_src", "interp_s16"):
            continue
        name = key[len("interp_"):]
        chroma = name.startswith("chroma")
        ins = s16 if name.endswith(("s16_pix", "s16_s16")) else src
        outt = np.int16 if name.endswith("s16") else o.pix
        fracs = list(range(0, 1024, 29)) if chroma else list(range(0, 256, 3)) + [8, 128, 136]
        i = 0
        for fi in ((0,) if chroma else (0, 1, 2)):
            for frac in fracs:
                b = np.zeros((4, 8), outt)
                getattr(o, name)(O.ptr(ins, 8 * ins.shape[1] + 8), ins.shape[1], O.ptr(b), 8, frac, 8, 4, fi)
                assert np.array_equal(b, g[key][i]), (name, fi, frac)
                i += 1
    t = g["quant_t"]
    for qp in range(52):
        p = O.orc_qparams()
        o.quant_params(qp, 4, 4, 0, qp & 1, qp & 2, p)
        q = np.zeros((16, 16), o.coef); r = np.zeros((16, 16), o.coef); nz = np.zeros(1, np.uint64)
        o.quant_inv_quant(O.ptr(q), O.ptr(t), O.ptr(r), 16, 16, 16, 4, 4, p.qmult, p.qadd, p.qshift, p.iqmult, p.iqadd,
                          p.iqshift, O.ptr(nz))
        assert np.array_equal(q, g["quant_q"][qp]) and np.array_equal(r, g["quant_r"][qp]) and nz[0] == g["quant_nz"][qp]
    off = 0
    for (w, h, m) in g["tr_cases"]:
        n = int(w * h)
        x = np.zeros((64, 64), o.coef); x[:h, :w] = g["tr_fin"][off:off + n].reshape(h, w)
        c = np.zeros((64, 64), o.coef); c[:h, :w] = g["tr_iin"][off:off + n].reshape(h, w)
        a = np.zeros((64, 64), o.coef); b = np.zeros((64, 64), o.coef)
        o.fdct_wxh(O.ptr(x), 64, O.ptr(a), 64, 0, int(w), int(h), int(m), 0, 1)
        o.idct_wxh(O.ptr(c), 64, O.ptr(b), 64, int(w), int(h), 0, 0, int(m), 1)
        assert np.array_equal(a[:h, :w].ravel(), g["tr_fout"][off:off + n]), (w, h, m)
        assert np.array_equal(b[:h, :w].ravel(), g["tr_iout"][off:off + n]), (w, h, m)
        off += n
    refp, inp = g["subpel_ref"], g["subpel_in"]
    pad = 24
    for mvx, mvy, ox, oy, oc in g["subpel_io"]:
        io = O.orc_me_io(int(mvx), int(mvy), 0x7FFFFFF0, 0)
        o.full_subpel_me(O.ptr(inp), 16, O.ptr(refp, pad * refp.shape[1] + pad), refp.shape[1], 16, 16, 1, -1, 57,
                         -10, -10, 10, 10, io)
        assert (io.best_mvx, io.best_mvy, io.best_cost) == (ox, oy, oc)


@pytest.mark.parametrize("bd", (8, 10))
def test_golden_dep_quant(bd):
    """Dependent quantisation: the reference's own outputs and tables (made by
    make_golden.py dq from h266_dep_quant.c compiled in place) against the oracle."""
    import ctypes as C
    g = np.load(os.path.join(GOLD, f"ref_dq_{bd}bit.npz"))
    o = O.oracle(bd)
    out = (C.c_uint32 * 2)()
    for s in range(256):
        o.dq_frac_bits(s, C.addressof(out))
        assert (out[0], out[1]) == tuple(g["frac_bits"][2 * s:2 * s + 2]), s
    assert [o.dq_rice_bits(k, n) for k in range(4) for n in range(32)] == list(g["rice_bits"])
    assert [o.dq_last_group(p) for p in range(64)] == list(g["last_group"])
    i = 0
    for lg in range(4, 13):
        for qp in range(52):
            p = O.orc_dq_param()
            o.dq_params(qp, lg, C.byref(p))
            assert [getattr(p, f) for f, _ in O.orc_dq_param._fields_] == list(g["dq_param"][i]), (lg, qp)
            i += 1
    sets = g["sets"]
    off = 0
    for (w, h, stride, qp, comp, root, cs), nz_ref in zip(g["meta"], g["nz"]):
        n = int(h * stride)
        t = g["t"][off:off + n].reshape(h, stride).astype(o.coef)
        q = np.zeros((h, stride), o.coef); r = np.zeros((h, stride), o.coef); nz = np.zeros(1, np.uint64)
        ctx = np.ascontiguousarray(sets[cs])
        o.dep_quant(O.ptr(t), int(stride), int(w), int(h), int(qp), int(comp), ctx.ctypes.data, int(root),
                    O.ptr(q), O.ptr(r), nz.ctypes.data)
        assert np.array_equal(q.ravel(), g["q"][off:off + n]), (w, h, qp, comp, root)
        assert np.array_equal(r.ravel(), g["r"][off:off + n]), (w, h, qp, comp, root)
        assert nz[0] == nz_ref
        off += n


@pytest.mark.parametrize("bd", (8, 10))
def test_golden_bilinear(bd):
    """Bilinear DMVR prediction: the reference's outputs (make_golden.py bili)."""
    g = np.load(os.path.join(GOLD, f"ref_bili_{bd}bit.npz"))
    o = O.oracle(bd)
    src = g["src"]
    for (w, h) in ((16, 8), (4, 4), (128, 4)):
        want = g[f"out_{w}x{h}"]
        i = 0
        for variant in range(4):
            for frac in list(range(0, 256, 5)) + [15, 240, 255]:
                b = np.zeros((h, w + 4), np.int16)
                o.bili_interp(variant, O.ptr(src, 2 * src.shape[1] + 2), src.shape[1], O.ptr(b), w + 4, frac, w, h)
                assert np.array_equal(b, want[i]), (w, h, variant, frac)
                i += 1
