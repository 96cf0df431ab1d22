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
