"""Generate tests/golden/reference_kats.npz from the REFERENCE's own render-layer
headers compiled for the host (oracle/_ref/libpupil_ref.so, built by
`make -C oracle ref` from the PupilOptixLab tree).

The reference has no tests and no fixtures of its own; these vectors are
its material, Fresnel, GGX, sampling, random-stream, emitter and curve code
run on seeded inputs.  Run once in a container that holds the reference tree:

    make -C oracle ref && python tests/golden/make_golden.py

The script is deterministic (numpy PCG64 seeds below).
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent / "reference_kats.npz"


def P(a):
    return a.ctypes.data_as(C.c_void_p)


def unit(v):
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def random_bsdfs(rng, n):
    b = np.zeros((n, 16), np.float32)
    b[:, 0] = np.repeat(np.arange(1, 8), (n + 6) // 7)[:n]
    b[:, 1] = rng.uniform(0.02, 0.8, n)
    b[:, 2] = rng.uniform(0.6, 2.4, n)  # eta, both sides of 1
    b[:, 3] = rng.uniform(0.3, 0.7, n)
    b[:, 4] = rng.uniform(0.05, 0.95, n)
    b[:, 5] = rng.integers(0, 2, n)
    b[:, 6:15] = rng.uniform(0.02, 0.98, (n, 9))
    cond = (b[:, 0] == 4) | (b[:, 0] == 5)
    b[cond, 9:12] = rng.uniform(0.1, 2.0, (cond.sum(), 3))   # eta
    b[cond, 12:15] = rng.uniform(1.0, 5.0, (cond.sum(), 3))  # k
    return b


def directions(rng, n, upper=0.75):
    v = unit(rng.normal(size=(n, 3)))
    up = rng.uniform(size=n) < upper
    v[:, 2] = np.where(up, np.abs(v[:, 2]), -np.abs(v[:, 2]))
    # edge cases: normal incidence, grazing, exactly tangent
    k = n // 16
    v[:k] = [0.0, 0.0, 1.0]
    v[k:2 * k] = unit(np.stack([np.ones(k), np.zeros(k), np.full(k, 1e-3)], 1))
    v[2 * k:3 * k] = unit(np.stack([rng.normal(size=k), rng.normal(size=k), np.zeros(k)], 1))
    return v.astype(np.float32)


def main():
    ref = oracle.load_ref()
    if ref is None:
        raise SystemExit("oracle/_ref/libpupil_ref.so not built (make -C oracle ref)")
    rng = np.random.default_rng(20240601)
    g = {}

    n = 1400
    b = random_bsdfs(rng, n)
    wo = directions(rng, n)
    wi = directions(rng, n)
    rng.shuffle(wi)
    f = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    ref.ref_bsdf_eval(P(b), P(wo), P(wi), P(f), P(pdf), n)
    g.update(eval_bsdf=b, eval_wo=wo, eval_wi=wi, eval_f=f, eval_pdf=pdf)

    b2 = random_bsdfs(rng, n)
    wo2 = directions(rng, n, upper=0.85)
    seeds = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    s_out = seeds.copy()
    wi2 = np.zeros((n, 3), np.float32)
    f2 = np.zeros((n, 3), np.float32)
    pdf2 = np.zeros(n, np.float32)
    typ = np.zeros(n, np.uint32)
    ref.ref_bsdf_sample(P(b2), P(wo2), P(s_out), P(wi2), P(f2), P(pdf2), P(typ), n)
    g.update(sample_bsdf=b2, sample_wo=wo2, sample_seed=seeds, sample_wi=wi2, sample_f=f2, sample_pdf=pdf2,
             sample_type=typ, sample_seed_out=s_out)

    pix = np.array([0, 1, 2, 255, 65535, 123456, 2073599, 4294967295], np.uint32)
    sd = np.array([0, 1, 7, 63, 1000, 12345, 4294967295, 42], np.uint32)
    streams = np.zeros((len(pix), 64), np.float32)
    for i, (p_, s_) in enumerate(zip(pix, sd)):
        ref.ref_rng_stream(int(p_), int(s_), 64, P(streams[i]))
    g.update(rng_pixel=pix, rng_seed=sd, rng_stream=streams)

    m = 512
    fin = np.stack([rng.uniform(1.0, 2.5, m), rng.uniform(-1, 1, m)], 1).astype(np.float32)
    fin[:8, 1] = [0.0, 1.0, -1.0, 1e-4, -1e-4, 0.5, -0.5, 0.2]
    fout = np.zeros((m, 2), np.float32)
    ref.ref_fresnel_dielectric(P(fin), P(fout), m)
    cin = np.stack([rng.uniform(0.1, 3, m), rng.uniform(0.5, 6, m), rng.uniform(0, 1, m)], 1).astype(np.float32)
    cout = np.zeros(m, np.float32)
    ref.ref_fresnel_conductor(P(cin), P(cout), m)
    din = rng.uniform(0.4, 3.0, m).astype(np.float32)
    dout = np.zeros(m, np.float32)
    ref.ref_fresnel_diffuse(P(din), P(dout), m)
    g.update(fresnel_in=fin, fresnel_out=fout, conductor_in=cin, conductor_out=cout, fdr_in=din, fdr_out=dout)

    gin = np.zeros((m, 9), np.float32)
    gin[:, 0:3] = directions(rng, m, upper=1.0)
    gin[:, 3:6] = unit(np.abs(rng.normal(size=(m, 3))) * [1, 1, 3])
    gin[:, 6] = rng.uniform(0.02, 0.9, m)
    gin[:, 7:9] = rng.uniform(0, 1, (m, 2))
    gout = np.zeros((m, 7), np.float32)
    ref.ref_ggx(P(gin), P(gout), m)
    g.update(ggx_in=gin, ggx_out=gout)

    sin_ = np.zeros((m, 8), np.float32)
    sin_[:, 0:2] = rng.uniform(0, 1, (m, 2))
    sin_[:, 2:5] = unit(rng.normal(size=(m, 3)))
    sin_[:, 5:8] = unit(rng.normal(size=(m, 3)))
    sin_[:4, 2:5] = [[0, 0, 1], [0, 0, -1], [1, 0, 0], [0, -1, 0]]
    sout = np.zeros((m, 20), np.float32)
    ref.ref_sampling(P(sin_), P(sout), m)
    g.update(sampling_in=sin_, sampling_out=sout)

    # emitters: one triangle, one sphere, one constant environment
    tri = np.array([5.0, 4.0, 3.0, 0.0,
                    -0.5, 2.0, -0.5, 0.0, -1.0, 0.0, 0.0, 0.0,
                    0.5, 2.0, -0.5, 0.0, -1.0, 0.0, 1.0, 0.0,
                    0.0, 2.0, 0.5, 0.0, -1.0, 0.0, 0.5, 1.0], np.float32)
    tri[3] = 0.5  # area of the triangle above
    sph = np.array([10.0, 10.0, 10.0, 4 * np.pi * 0.25, 1.0, 3.0, -1.0, 0.5], np.float32)
    env = np.array([0.5, 0.6, 0.7], np.float32)
    ein = np.zeros((m, 8), np.float32)
    ein[:, 0:3] = rng.uniform(-1, 1, (m, 3)) * [1, 0.5, 1]
    ein[:, 3:6] = unit(rng.normal(size=(m, 3)) + [0, 1.0, 0])
    ein[:, 6:8] = rng.uniform(0, 1, (m, 2))
    outs = []
    for kind, params in ((1, tri), (2, sph), (3, env)):
        o = np.zeros((m, 12), np.float32)
        ref.ref_emitter_sample(kind, P(params), P(ein), P(o), m)
        outs.append(o)
    g.update(emit_tri=tri, emit_sphere=sph, emit_env=env, emit_in=ein, emit_tri_out=outs[0],
             emit_sphere_out=outs[1], emit_env_out=outs[2])

    probs = (rng.uniform(0.1, 1.0, 37) / 60.0).astype(np.float32)
    pv = rng.uniform(0, 1, 2000).astype(np.float32)
    pv[:5] = [0.0, probs[0], probs[0] + probs[1], 1.0, 0.9999999]
    sel_env = np.zeros(2000, np.int32)
    sel_noenv = np.zeros(2000, np.int32)
    ref.ref_select_emitter(P(probs), len(probs), 1, P(pv), P(sel_env), 2000)
    ref.ref_select_emitter(P(probs), len(probs), 0, P(pv), P(sel_noenv), 2000)
    g.update(select_probs=probs, select_p=pv, select_env=sel_env, select_noenv=sel_noenv)

    # environment map: a 24 x 12 map with a bright patch, rotated 30 degrees
    # about y, sampled (xi drawn below the last row's interval: the reference
    # reads past its tables for that row) and evaluated in random directions
    import oracle as orc
    ew, eh = 24, 12
    emap = rng.uniform(0.05, 0.5, (eh, ew, 4)).astype(np.float32)
    emap[3:5, 15:18, :3] = [[30.0, 25.0, 20.0]]
    emap[:, :, 3] = 1.0
    ang = np.radians(30.0)
    tw = np.array([[np.cos(ang), 0, np.sin(ang)], [0, 1, 0], [-np.sin(ang), 0, np.cos(ang)]], np.float32)
    tl = np.linalg.inv(tw.astype(np.float64)).astype(np.float32)
    _, tables = orc.envmap(0, emap, 1.5, tw, tl, np.zeros((1, 2), np.float32))
    row_cdf = tables[:eh + 1].copy()
    col_cdf = tables[eh + 1:eh + 1 + (ew + 1) * eh].copy()
    row_weight = tables[eh + 1 + (ew + 1) * eh:eh + 1 + (ew + 1) * eh + eh].copy()
    norm = float(tables[-1])
    xi = rng.uniform(0, 1, (m, 2)).astype(np.float32)
    xi[:, 0] *= row_cdf[eh - 1]
    xi[:4] = [[0.0, 0.0], [row_cdf[3], 0.5], [0.5, 0.0], [row_cdf[eh - 1], 0.999]]
    es = np.zeros((m, 7), np.float32)
    ref.ref_envmap(0, P(emap), ew, eh, 1.5, P(tw), P(tl), P(row_cdf), P(col_cdf), P(row_weight), norm, P(xi), P(es), m)
    ev_in = np.zeros((m, 6), np.float32)
    ev_in[:, 0:3] = rng.uniform(-2, 2, (m, 3))
    ev_in[:, 3:6] = unit(rng.normal(size=(m, 3)))
    ev = np.zeros((m, 4), np.float32)
    ref.ref_envmap(1, P(emap), ew, eh, 1.5, P(tw), P(tl), P(row_cdf), P(col_cdf), P(row_weight), norm, P(ev_in),
                   P(ev), m)
    g.update(envmap_pixels=emap, envmap_tw=tw, envmap_tl=tl, envmap_xi=xi, envmap_sample=es, envmap_eval_in=ev_in,
             envmap_eval=ev)

    # curve interpolators and SurfaceNormal (render/curve.h) for the four
    # curve types: random control points (radius in w), u with the end values
    # 0 and 1 (cap normals, the cubic derivative's triple-knot nudge), hit
    # points slightly off the swept circle at u
    nc = 256
    for ct in range(4):
        ctrl = np.zeros((nc, 4, 4), np.float32)
        ctrl[:, :, :3] = rng.uniform(-1, 1, (nc, 4, 3))
        ctrl[:, :, 3] = rng.uniform(0.01, 0.2, (nc, 4))
        u = rng.uniform(0, 1, nc).astype(np.float32)
        u[:4] = [0.0, 1.0, 0.5, 1e-7]
        probe = np.zeros((nc, 15), np.float32)
        ref.ref_curve(ct, P(ctrl), P(u), P(np.zeros((nc, 3), np.float32)), P(probe), nc)
        vel = probe[:, 4:7].astype(np.float64)
        side = rng.normal(size=(nc, 3))
        side -= (np.sum(side * vel, 1) / np.maximum(np.sum(vel * vel, 1), 1e-12))[:, None] * vel
        side /= np.linalg.norm(side, axis=1, keepdims=True)
        ps = (probe[:, 0:3] + side * (probe[:, 3:4] * rng.uniform(0.98, 1.02, (nc, 1)))).astype(np.float32)
        out = np.zeros((nc, 15), np.float32)
        ref.ref_curve(ct, P(ctrl), P(u), P(ps), P(out), nc)
        g.update({f"curve{ct}_ctrl": ctrl, f"curve{ct}_u": u, f"curve{ct}_ps": ps, f"curve{ct}_out": out})

    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(g)} arrays)")


if __name__ == "__main__":
    main()
