"""Generate the golden fixtures in tests/golden/ from the reference's own C.

Runs in the container that has the xin26x source tree: it builds
oracle/_ref/libxinref{8,10}.so (the reference's open hot-path C compiled in
place, oracle/Makefile target ``ref``) and records seeded inputs with that
library's outputs.  tests/test_oracle_golden.py replays the inputs through
the oracle anywhere (no reference tree needed) and requires identical output.

    python tests/golden/make_golden.py [core|dq|bili]
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def scan_cg(wcg, hcg):
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


def make(bd):
    O.build(ref=True)
    r = O.reference(bd)
    o = O.oracle(bd)
    rng = np.random.default_rng(20260 + bd)
    g = {}
    # interpolation: one 16x8 block per (function, filter index, phase subset)
    src = rng.integers(0, r.max_pix + 1, size=(4 + 16, 8 + 16)).astype(r.pix)
    s16 = rng.integers(-8192, 8192, size=(4 + 16, 8 + 16)).astype(np.int16)
    g["interp_src"] = src
    g["interp_s16"] = s16
    for name in ["luma_hor", "luma_vet", "luma_hv", "luma_hor_s16", "luma_vet_s16", "luma_hv_s16", "luma_vet_s16_pix",
                 "luma_vet_s16_s16", "chroma_hor", "chroma_vet", "chroma_hv", "chroma_hor_s16", "chroma_vet_s16",
                 "chroma_hv_s16", "chroma_vet_s16_pix", "chroma_vet_s16_s16"]:
        chroma = name.startswith("chroma")
        ins = s16 if name.endswith(("s16_pix", "s16_s16")) else src
        outt = np.int16 if name.endswith("s16") else r.pix
        fracs = list(range(0, 1024, 29)) if chroma else list(range(0, 256, 3)) + [8, 128, 136]
        res = []
        for fi in ((0,) if chroma else (0, 1, 2)):
            for frac in fracs:
                b = np.zeros((4, 8), outt)
                getattr(r, name)(O.ptr(ins, 8 * ins.shape[1] + 8), ins.shape[1], O.ptr(b), 8, frac, 8, 4, fi)
                res.append(b)
        g[f"interp_{name}"] = np.stack(res)
    # quantiser
    t = np.clip(rng.laplace(0, 400, size=(16, 16)), -32768, 32767).astype(r.coef)
    g["quant_t"] = t
    qo, ro, nzo = [], [], []
    for qp in range(0, 52):
        p = O.orc_qparams()
        o.quant_params(qp, 4, 4, 0, qp & 1, qp & 2, p)
        q = np.zeros((16, 16), r.coef); rr = np.zeros((16, 16), r.coef); nz = np.zeros(1, np.uint64)
        r.quant_inv_quant(O.ptr(q), O.ptr(t), O.ptr(rr), 16, 16, 16, 4, 4, p.qmult, p.qadd, p.qshift, p.iqmult, p.iqadd,
                          p.iqshift, O.ptr(nz))
        qo.append(q); ro.append(rr); nzo.append(nz[0])
    g["quant_q"], g["quant_r"], g["quant_nz"] = np.stack(qo), np.stack(ro), np.array(nzo, np.uint64)
    # transforms through the reference's 2-D wrappers (all MTS types, 4..32 and DCT2 64)
    cases = [(w, h, m) for (w, h) in [(4, 4), (8, 8), (16, 16), (32, 32), (4, 16), (32, 8)] for m in range(6)]
    cases += [(64, 64, 0), (64, 16, 0), (8, 64, 0)]
    fres, ires, fin, iin = [], [], [], []
    lim = (1 << bd) - 1
    for (w, h, m) in cases:
        x = rng.integers(-lim, lim + 1, size=(64, 64)).astype(r.coef)
        c = np.clip(rng.laplace(0, 300, size=(64, 64)), -32768, 32767).astype(r.coef)
        c[32:, :] = 0
        c[:, 32:] = 0
        a = np.zeros((64, 64), r.coef)
        b = np.zeros((64, 64), r.coef)
        r.fdct_wxh(O.ptr(x), 64, O.ptr(a), 64, 0, w, h, m, 0, 1)
        r.idct_wxh(O.ptr(c), 64, O.ptr(b), 64, w, h, 0, 0, m, 1)
        for lst, arr in ((fin, x), (iin, c), (fres, a), (ires, b)):
            lst.append(arr[:h, :w].ravel())
    g["tr_cases"] = np.array(cases, np.int32)
    g["tr_fin"], g["tr_fout"], g["tr_iin"], g["tr_iout"] = map(np.concatenate, (fin, fres, iin, ires))
    # sub-pel search
    pad = 24
    refp = rng.integers(0, r.max_pix + 1, size=(16 + 2 * pad, 16 + 2 * pad)).astype(r.pix)
    inp = refp[pad + 1:pad + 17, pad + 2:pad + 18].copy()
    g["subpel_ref"], g["subpel_in"] = refp, inp
    sp = []
    for mvx in range(-6, 7, 3):
        for mvy in range(-6, 7, 3):
            io = np.array([mvx, mvy, 0x7FFFFFF0], np.int32)
            r.full_subpel_me_io(O.ptr(inp), 16, O.ptr(refp, pad * refp.shape[1] + pad), refp.shape[1], 16, 16, 1, -1, 57,
                                -10, -10, 10, 10, O.ptr(io))
            sp.append([mvx, mvy, io[0], io[1], io[2]])
    g["subpel_io"] = np.array(sp, np.int64)
    np.savez_compressed(os.path.join(OUT, f"ref_golden_{bd}bit.npz"), **g)
    print("wrote", os.path.join(OUT, f"ref_golden_{bd}bit.npz"))


def make_dq(bd):
    """Dependent quantisation: seeded blocks of every size 4..64 and component,
    QP 0..51, root cbf on and off, with strided layouts, through the reference's
    Xin266DepQuant; plus the reference's rate / Rice / group-index tables and
    trellis parameters that the oracle derives from formulas."""
    import ctypes as C
    from xin26x_gb300 import synth as S
    O.build(ref=True)
    r = O.reference(bd)
    rng = np.random.default_rng(4100 + bd)
    sets = S.contexts(rng, 8)
    sizes = [(w, h) for w in (4, 8, 16, 32, 64) for h in (4, 8, 16, 32, 64)]
    meta, tin, qout, rout, nzs = [], [], [], [], []
    for i in range(8 * len(sizes)):
        w, h = sizes[i % len(sizes)]
        stride = w + int(rng.choice([0, 0, 4, 12]))
        qp, comp, root, cs = int(rng.integers(0, 52)), int(rng.integers(0, 3)), int(rng.integers(0, 2)), int(rng.integers(0, 8))
        t = np.zeros((h, stride), r.coef)
        t[:, :w] = S.coefficients(rng, w, h, bd)
        q = np.zeros((h, stride), r.coef); rr = np.zeros((h, stride), r.coef); nz = np.zeros(1, np.uint64)
        ctx = np.ascontiguousarray(sets[cs])
        r.dep_quant(O.ptr(t), stride, w, h, qp, comp, ctx.ctypes.data, root, O.ptr(q), O.ptr(rr), nz.ctypes.data)
        meta.append([w, h, stride, qp, comp, root, cs])
        tin.append(t.ravel()); qout.append(q.ravel()); rout.append(rr.ravel()); nzs.append(nz[0])
    g = {"meta": np.array(meta, np.int32), "t": np.concatenate(tin), "q": np.concatenate(qout),
         "r": np.concatenate(rout), "nz": np.array(nzs, np.uint64), "sets": sets}
    g["frac_bits"] = np.ctypeslib.as_array((C.c_uint32 * 512).in_dll(r.lib, "cabacbinFracBits")).copy()
    g["rice_bits"] = np.ctypeslib.as_array((C.c_int32 * 128).in_dll(r.lib, "goRiceBits")).copy()
    g["rice_par"] = np.ctypeslib.as_array((C.c_uint32 * 32).in_dll(r.lib, "auiGoRiceParsCoeff")).copy()
    g["last_group"] = np.ctypeslib.as_array((C.c_uint32 * 64).in_dll(r.lib, "lastSigXYGroupIdx")).copy()
    par = []
    for lg in range(4, 13):
        for qp in range(52):
            d = O.xin_dp_param()
            r.dq_param_ref(qp, lg, C.byref(d))
            par.append([getattr(d, f) for f, _ in O.orc_dq_param._fields_])
    g["dq_param"] = np.array(par, np.int64)
    np.savez_compressed(os.path.join(OUT, f"ref_dq_{bd}bit.npz"), **g)
    print("wrote", os.path.join(OUT, f"ref_dq_{bd}bit.npz"))


def make_bili(bd):
    """Bilinear DMVR prediction (h266_bilinear_filter.c) through the reference:
    four variants, 55 phases spread over all 256, on a 16x8, a 4x4 and a 128x4 block."""
    O.build(ref=True)
    r = O.reference(bd)
    rng = np.random.default_rng(5200 + bd)
    src = rng.integers(0, r.max_pix + 1, size=(12, 144)).astype(r.pix)
    g = {"src": src}
    for (w, h) in ((16, 8), (4, 4), (128, 4)):
        res = []
        for variant in range(4):
            for frac in list(range(0, 256, 5)) + [15, 240, 255]:
                b = np.zeros((h, w + 4), np.int16)
                r.bili_interp(variant, O.ptr(src, 2 * src.shape[1] + 2), src.shape[1], O.ptr(b), w + 4, frac, w, h)
                res.append(b)
        g[f"out_{w}x{h}"] = np.stack(res)
    np.savez_compressed(os.path.join(OUT, f"ref_bili_{bd}bit.npz"), **g)
    print("wrote", os.path.join(OUT, f"ref_bili_{bd}bit.npz"))


if __name__ == "__main__":
    what = sys.argv[1:] or ["all"]
    for bd in (8, 10):
        if "all" in what or "core" in what:
            make(bd)
        if "all" in what or "dq" in what:
            make_dq(bd)
        if "all" in what or "bili" in what:
            make_bili(bd)
