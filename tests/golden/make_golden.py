"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference's own classes, compiled unmodified from its sources with
the oracle shims (``make -C oracle ref``), through tests/oracle_lib.RefChain,
and writes small .npz files.  The reference ships no golden vectors or
known-answer tests; these pin the oracle restatement (tests/test_oracle_golden.py)
on machines where the reference sources are absent.

    python tests/golden/make_golden.py
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import oracle_lib as ol  # noqa: E402

PHI = 0.25 * math.pi


def trace_arrays(t):
    return {"v1": t["v1"].astype(np.int16), "v2": t["v2"].astype(np.int16), "kind": t["kind"].astype(np.int8),
            "accepted": t["accepted"].astype(np.int8), "ratio": t["ratio"], "u4": t["u"][:, 3]}


def main():
    if not ol.reference_available():
        sys.exit("reference build missing: run `make -C oracle ref` where the reference sources exist")
    out = {}

    # 1. Phi tables (StagFluxWaveFunction::matrix_element via WaveFunction::MatEl)
    for L, neel, ne, bc in [(4, 0.1, 0.0, (1.0, 1.0)), (6, 0.05, 0.0, (1.0, 1.0)), (8, 0.1, 0.5, (1.0, 0.0))]:
        r = ol.RefChain(L, PHI, neel, neel_exp=ne, bc=bc)
        d = {"L": L, "neel": neel, "neel_exp": ne, "bc": np.array(bc), "phi": PHI}
        for fl in (0, 1):
            t = r.phi_table(fl)
            d["phi%d" % fl] = t if L < 8 else t[:8]
        d["nbr"] = r.neighbours()
        d["orb0"] = r.orbitals(0)
        np.savez_compressed(os.path.join(HERE, "phi_L%d.npz" % L), **d)
        out["phi_L%d" % L] = True

    # 2. Ground state L=8 trace from the random start (seed 1234, walker 0)
    r = ol.RefChain(8, PHI, 0.1, seed=1234, walker=0)
    assert r.random_start() == 0
    start = r.config()
    am0, ae0 = r.amp()
    inv0 = r.inverse(0)
    t = r.walk(4000, trace=True)
    am, ae = r.amp()
    np.savez_compressed(os.path.join(HERE, "gs_L8_trace.npz"), start=start, amp0=np.array([am0.real, am0.imag, ae0]),
                        inv0_up=inv0, final=r.config(), amp=np.array([am.real, am.imag, ae]),
                        inv_up=r.inverse(0), **trace_arrays(t))

    # 3. Measurements: L=8 ProjHeis+StagMagnZ after thermalisation, L=4 all three
    r = ol.RefChain(8, PHI, 0.1, seed=5, walker=0)
    r.random_start()
    r.walk(200 * 64)
    r.walk(64 * 30, meas=64, mask=ol.MEAS_PROJHEIS | ol.MEAS_STAGMAGN)
    pj, n1 = r.projheis()
    sm, n2 = r.stagmagn()
    # a seed whose first random start is non-singular: the reference's retry
    # keeps stale occupancies (State::InitFock does not clear m_fock)
    for seed4 in range(6, 60):
        r4 = ol.RefChain(4, PHI, 0.1, seed=seed4, walker=2)
        r4.random_start()
        if int(r4.config().sum()) == 8:
            break
    r4.walk(200 * 16)
    r4.walk(16 * 40, meas=16, mask=7)
    pj4, _ = r4.projheis()
    sm4, _ = r4.stagmagn()
    ss4, nss = r4.statspin()
    np.savez_compressed(os.path.join(HERE, "gs_meas.npz"), pj8=pj, n8=n1, sm8=sm, pj4=pj4, sm4=sm4, ss4=ss4, n4=nss,
                        seed4=seed4,
                        final8=r.config(), final4=r4.config())

    # 4. Re-inversion cadence (every L^2 accepted exchanges)
    r = ol.RefChain(8, PHI, 0.1, seed=11, walker=0)
    r.random_start()
    t = r.walk(3000, reinv_every=64, trace=True)
    np.savez_compressed(os.path.join(HERE, "gs_L8_reinv.npz"), final=r.config(), reinv=r.counts()[3], **trace_arrays(t))

    # 5. Transverse exciton channel
    for L, q, steps in [(4, (2, 2), 2000), (8, (4, 4), 1500)]:
        r = ol.RefChain(L, PHI, 0.1, channel=ol.TRANS, q=q, seed=7, walker=3)
        assert r.random_start() == 0
        st0 = r.current_state()
        t = r.walk(steps, trace=True)
        r.walk(L * L * 6, meas=L * L, mask=ol.MEAS_PROJHEIS)
        pj, n = r.projheis()
        am, ae = r.amp()
        np.savez_compressed(os.path.join(HERE, "trans_L%d.npz" % L), q=np.array(q), state0=st0,
                            state=r.current_state(), final=r.config(), amp=np.array([am.real, am.imag, ae]),
                            pj=pj, n=n, **trace_arrays(t))

    # 6. VirtUpdate bond-swap ratios for a fixed configuration
    r = ol.RefChain(8, PHI, 0.1, seed=3, walker=0)
    r.random_start()
    up = r.config().astype(bool)
    L = 8
    hops = []
    for x in range(L):
        for y in range(L):
            a = y * L + x
            for b in (((y + 1) % L) * L + x, y * L + (x + 1) % L):
                if up[a] != up[b]:
                    u, dn = (a, b) if up[a] else (b, a)
                    hops.append((u, dn, dn, u))
    hops = np.array(hops, dtype=np.int32)
    qm, qe = r.virt_update(hops)
    am, ae = r.amp()
    np.savez_compressed(os.path.join(HERE, "gs_L8_virt.npz"), config=r.config(), hops=hops, qm=qm, qe=qe,
                        amp=np.array([am.real, am.imag, ae]))
    long_exciton()
    print("golden fixtures written to", HERE)


def long_exciton():
    """7. Longitudinal exciton channel (StagFluxLongExciton): states two
    orbital hops apart in one flavour; q = (0, 0) adds the ground state."""
    for L, q, steps in [(4, (2, 0), 1500), (4, (0, 0), 1500)]:
        r = ol.RefChain(L, PHI, 0.1, channel=ol.LONG, q=q, seed=7, walker=3)
        assert r.random_start() == 0
        st0 = r.current_state()
        t = r.walk(steps, trace=True)
        r.walk(L * L * 6, meas=L * L, mask=ol.MEAS_PROJHEIS)
        pj, n = r.projheis()
        am, ae = r.amp()
        np.savez_compressed(os.path.join(HERE, "long_L%d_q%d%d.npz" % (L, q[0], q[1])), q=np.array(q), state0=st0,
                            state=r.current_state(), final=r.config(), amp=np.array([am.real, am.imag, ae]),
                            pj=pj, n=n, **trace_arrays(t))


if __name__ == "__main__":
    main()
