"""Regenerate the golden vectors in this folder from the reference imager's own CPU code.

The reference (PaCER-BLINK-Project/imager) has no runnable test data here, so its CPU sources
(src/corrections.cpp, src/pacer_imager.cpp, src/utils.cpp) are compiled against the stand-in
headers in oracle/ref_shim (``make -C oracle ref``) and run on small seeded inputs.  The outputs
pin the oracle: tests/test_oracle_golden.py checks the oracle against these files on any host,
without the reference checkout.

Run from the repository root:  python tests/golden/make_golden.py
(the reference checkout's src/ is found through BGI_REFERENCE_SRC, or as a checkout named
"reference" beside this repository).
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from imager_gb300 import synth  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# obsInfo fields for the cotter-compatible channel frequencies (src/pacer_imager.cpp:528-555)
COARSE_BW_MHZ, COARSE_CHANNEL, FREQ_RES_MHZ, N_AVG = 1.28, 118, 0.04, 4


def ref_run(obs, vis, n_pixels, pol, min_uv=-1000.0, weighting=b"N", geom=1, cable=1,
            flagged=(3,), freq_override_mhz=-1.0, osf=2.0, kernel=0):
    ref = O.ref_library()
    ref.ref_set_kernel_size(int(kernel))  # m_nConvolvingKernelSize (0: nearest neighbour)
    T, Cn, nb = vis.shape[:3]
    n_ant = obs.n_ant
    npix = n_pixels * n_pixels * T * Cn
    vout = np.zeros(vis.size, np.float32)
    g = np.zeros(npix * 2, np.float32)
    c = np.zeros(npix, np.float32)
    im = np.zeros(npix * 2, np.float32)
    sc = np.zeros(4)
    fa = np.asarray(list(flagged) or [0], np.int32)
    ref.ref_run(np.ascontiguousarray(vis, np.float32).reshape(-1), T, Cn, n_ant,
                np.ascontiguousarray(obs.u[0]), np.ascontiguousarray(obs.v[0]),
                np.ascontiguousarray(obs.w[0]), obs.cable, fa, len(flagged), FREQ_RES_MHZ, N_AVG,
                COARSE_BW_MHZ, COARSE_CHANNEL, freq_override_mhz, n_pixels, osf, min_uv, pol,
                weighting, geom, cable, vout, g, c, im, sc)
    shape = (T, Cn, n_pixels, n_pixels)
    return dict(vis_out=vout.reshape(vis.shape), grids=g.reshape(shape + (2,)),
                counters=c.reshape(shape), images=im.reshape(shape + (2,)), scalars=sc)


def main():
    O.build(ref=True)
    if O.ref_library() is None:
        raise SystemExit("reference build missing: set BGI_REFERENCE_SRC to the reference checkout's src/")
    cases = {}

    # 1) corrections on their own (src/corrections.cpp), one UVW set
    obs = synth.small(seed=11, n_ant=20, n_intervals=2, n_channels=3, per_interval_uvw=False)
    vis = obs.vis_f32().copy()
    geo = vis.copy().reshape(-1)
    O.ref_library().ref_apply_geometric_cpu(geo, 2, 3, obs.n_ant, obs.w[0].copy(), obs.freqs)
    cab = vis.copy().reshape(-1)
    O.ref_library().ref_apply_cable_cpu(cab, 2, 3, obs.n_ant, obs.cable, obs.freqs)
    np.savez_compressed(os.path.join(OUT, "corrections.npz"), vis=vis, w=obs.w[0], cable=obs.cable,
                        freqs=obs.freqs, after_geometric=geo.reshape(vis.shape),
                        after_cable=cab.reshape(vis.shape))

    # 2) CPacerImager::run() end to end, four polarisations, two image sizes
    obs = synth.small(seed=12, n_ant=20, n_intervals=2, n_channels=3, per_interval_uvw=False)
    vis = obs.vis_f32().copy()
    freqs = np.array([O.library().bgo_channel_frequency_hz(FREQ_RES_MHZ, N_AVG, COARSE_BW_MHZ,
                                                           COARSE_CHANNEL, ch, 1)
                      for ch in range(vis.shape[1])])
    for pol_name, pol in O.POL.items():
        cases[f"run_{pol_name}_32"] = (obs, vis, 32, pol, dict())
    cases["run_XX_48"] = (obs, vis, 48, 0, dict())
    # 3) a positive min_uv cut
    cases["run_XX_32_minuv"] = (obs, vis, 32, 0, dict(min_uv=20.0))
    # 4) NaN, inf and |x| >= 1e12 values are skipped (src/pacer_imager.cpp:327-329)
    bad = vis.copy()
    bad[0, 0, 5, 0, 0] = np.nan
    bad[0, 1, 7, 0, 1] = np.inf
    bad[1, 2, 9, 0, 0] = 2e12
    bad[1, 0, 11, 3, 1] = np.nan
    cases["run_XX_32_bad"] = (obs, bad, 32, 0, dict(geom=0, cable=0))
    cases["run_YY_32_bad"] = (obs, bad, 32, 1, dict(geom=0, cable=0))
    # 5) single-frequency override (m_fFrequencyMHz, src/pacer_imager.cpp:454-457), no flags
    cases["run_I_32_fixedfreq"] = (obs, vis, 32, 2, dict(freq_override_mhz=159.375, flagged=()))
    # 6) uniform weighting: empty cells become 0/0 (src/pacer_imager.cpp:421-428)
    cases["run_XX_32_uniform"] = (obs, vis, 32, 0, dict(weighting=b"U"))
    # 7) Kaiser-Bessel convolution kernels (src/pacer_imager.cpp:378-403, 565-750); odd sizes,
    #    as an even size makes the reference write one element past its kernel vector
    cases["run_XX_32_kb7"] = (obs, vis, 32, 0, dict(kernel=7))
    cases["run_I_48_kb11"] = (obs, vis, 48, 2, dict(kernel=11))
    cases["run_V_32_kb5_minuv"] = (obs, vis, 32, 3, dict(kernel=5, min_uv=20.0))

    arrays = dict(u=obs.u[0], v=obs.v[0], w=obs.w[0], cable=obs.cable, vis=vis, vis_bad=bad,
                  freqs_cotter=freqs)
    for name, (o, x, n, pol, kw) in cases.items():
        r = ref_run(o, x, n, pol, **kw)
        for k, val in r.items():
            arrays[f"{name}__{k}"] = val
    meta = {name: dict(n_pixels=n, pol=pol, **{k: (v.decode() if isinstance(v, bytes) else v)
                                               for k, v in kw.items()})
            for name, (o, x, n, pol, kw) in cases.items()}
    arrays["meta"] = np.array(repr(meta))
    np.savez_compressed(os.path.join(OUT, "imager_run.npz"), **arrays)

    # 8) pointed-observation UVW with the reference's geometry routines (src/pacer_geometry.h)
    rng = np.random.default_rng(17)
    n_ant, T = 30, 3
    xyz = rng.uniform(-1500.0, 1500.0, (n_ant, 3))
    ang = [rng.uniform(0, 2 * np.pi, T) for _ in range(4)]  # ha2000, dec (below), lmst, lmst2000
    dec = rng.uniform(-1.2, 0.3, T)
    rmat = np.empty((T, 3, 3))
    for t in range(T):  # a small rotation, as the precession-nutation matrix is
        a, b, c = rng.uniform(-3e-3, 3e-3, 3)
        k = np.array([[0, -c, b], [c, 0, -a], [-b, a, 0]])
        rmat[t] = np.eye(3) + k + 0.5 * k @ k
    nb = n_ant * (n_ant + 1) // 2
    u, v, w = (np.empty((T, nb), np.float32) for _ in range(3))
    steps = np.empty((T, 17))
    O.ref_library().ref_pointed_uvw(np.ascontiguousarray(xyz).reshape(-1), n_ant, rmat.reshape(-1), ang[0], dec,
                                    ang[2], ang[3], T, u.reshape(-1), v.reshape(-1), w.reshape(-1), steps.reshape(-1))
    np.savez_compressed(os.path.join(OUT, "pointed_uvw.npz"), xyz=xyz, rmat=rmat, ha2000=ang[0], dec_aber=dec,
                        lmst=ang[2], lmst2000=ang[3], steps=steps, u=u, v=v, w=w)

    # 7) fft_shift known answers, computed by the reference's fft_shift (src/pacer_imager.cpp:110)
    shifts = {}
    for (ny, nx) in ((2, 2), (2, 3), (3, 3), (4, 6), (5, 4)):
        x = np.arange(ny * nx, dtype=np.complex64).reshape(ny, nx) * (1 + 0.5j)
        y = x.copy().view(np.float32).reshape(-1)
        O.ref_library().ref_fft_shift(y, nx, ny)
        shifts[f"in_{ny}x{nx}"] = x
        shifts[f"out_{ny}x{nx}"] = y.view(np.complex64).reshape(ny, nx)
    np.savez_compressed(os.path.join(OUT, "fft_shift.npz"), **shifts)
    print("golden vectors written to", OUT)


if __name__ == "__main__":
    main()
