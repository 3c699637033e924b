"""Generate the golden fixtures in tests/golden/ from the REFERENCE's own code.

The reference sources are compiled unchanged (oracle/build_ref.sh) into
oracle/_ref/libigapref.so and driven through its public set-up
(IGAPAssmInit), its SNES callbacks (Residual_iga / Tangent_iga), its
density integral (iga_intdensity, stored as HH) and, for the small cases, the
field callbacks on the plot lattice of iga_plotfield (the reference's basis,
inverse and field callback in a restated loop, since plotcore_iga.c does not
compile; stored as field / field_xq / field_X at FIELD_SCALE x the state).  The
fixtures are what the reference outputs for seeded inputs, so tests on a
machine without the reference tree still compare against the reference.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle as po  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def beam_problem(nelem, law, L=(4.0, 1.0, 1.0), perturb=False, **kw):
    bct, neu = po.clamp_bc((0,), 1, (0.0, 0.0, -1e-3))
    return po.Problem(nelem=nelem, L=L, law=law, perturb=perturb, bc_type=bct, neumann=neu, **kw)


# Small cases: full residual Vec and full AIJ matrix are stored.
FULL_CASES = {
    "g_static_2x2x2": dict(nelem=(2, 2, 2), law=po.LAW_GRADELAST, seed=11),
    "g_lingrad_4x2x2": dict(nelem=(4, 2, 2), law=po.LAW_LINGRAD, seed=12),
    "g_transient_3x2x2": dict(nelem=(3, 2, 2), law=po.LAW_GRADELASTTIME, seed=13, L=(1.0, 1.0, 1.0)),
}
# Larger cases: full residual, tangent summarised (pattern checksum, norm,
# sampled slots) to keep the fixtures small.
SUMMARY_CASES = {
    "g_static_beamtest_4x4x4": dict(nelem=(4, 4, 4), law=po.LAW_GRADELAST, seed=21,
                                    L=(1.0, 1.0, 1.0), perturb=True),
    "g_lingrad_8x2x2": dict(nelem=(8, 2, 2), law=po.LAW_LINGRAD, seed=22),
}
NSAMPLE = 4096
FIELD_NPPE = 2
FIELD_SCALE = 10.0  # large enough strains to reach every sector code


def main():
    if not po.ref_available():
        raise SystemExit("oracle/_ref/libigapref.so is required (run oracle/build_ref.sh)")
    for name, spec in {**FULL_CASES, **SUMMARY_CASES}.items():
        spec = dict(spec)
        seed = spec.pop("seed")
        prob = beam_problem(**spec)
        U = po.random_state(prob, seed)
        case = po.RefCase(prob)
        RR = case.residual(U)
        rowptr, cols, vals = case.tangent(U)
        meta = dict(nelem=np.array(prob.nelem), L=np.array(prob.L), law=prob.law,
                    perturb=int(prob.perturb), seed=seed, par=prob.params(),
                    bc_type=prob.bc_type, neumann=prob.neumann, U=U, RR=RR, HH=case.density(U))
        if name in FULL_CASES:
            meta.update(rowptr=rowptr, cols=cols, vals=vals)
            F, xq, X = case.field(FIELD_SCALE * U, FIELD_NPPE)
            meta.update(field_nppe=FIELD_NPPE, field_scale=FIELD_SCALE, field=F, field_xq=xq, field_X=X)
        else:
            rng = np.random.default_rng(seed)
            idx = np.sort(rng.choice(len(vals), NSAMPLE, replace=False))
            meta.update(rowptr=rowptr, cols_sum=np.int64(cols.astype(np.int64).sum()),
                        cols_wsum=np.int64((cols.astype(np.int64) * np.arange(len(cols)) % 1000003).sum()),
                        vals_norm=np.linalg.norm(vals), vals_sum=vals.sum(), sample_idx=idx,
                        sample_vals=vals[idx])
        np.savez_compressed(os.path.join(OUT, name + ".npz"), **meta)
        print(name, "ndof", case.ndof, "nnz", len(vals))

    # law-level known answers: seeded points, each law at its default params
    rng = np.random.default_rng(5)
    laws = {}
    for law in (po.LAW_GRADELAST, po.LAW_GRADELASTTIME, po.LAW_LINGRAD):
        par = np.zeros(9)
        po.ref().ref_law_default_par(law, par.ctypes.data_as(po._D))
        us, rrs, tts = [], [], []
        for _ in range(6):
            u = rng.uniform(-0.05, 0.05, 90)
            rr, tt = po.law_eval("ref", law, u, par)
            us.append(u); rrs.append(rr); tts.append(tt)
        laws[f"u_{law}"] = np.array(us)
        laws[f"rr_{law}"] = np.array(rrs)
        laws[f"tt_{law}"] = np.array(tts)
        laws[f"par_{law}"] = par
    np.savez_compressed(os.path.join(OUT, "laws.npz"), **laws)

    # quadrature and basis known answers
    quad = {}
    for n in (2, 3, 4, 5, 6):
        x = np.zeros(n); w = np.zeros(n)
        po.ref().ref_gauss_legendre(n, 0.0, 1.0, x.ctypes.data_as(po._D), w.ctypes.data_as(po._D))
        quad[f"x{n}"] = x
        quad[f"w{n}"] = w
    np.savez_compressed(os.path.join(OUT, "quadrature.npz"), **quad)

    # sanity value: 4x4x4 unit cube, gradelast, face 0 clamped, glibc
    # rand() seed 123456 scaled 0.01 (IGAPSolvRand, src/interface.c:261-269)
    print("done")


if __name__ == "__main__":
    main()
