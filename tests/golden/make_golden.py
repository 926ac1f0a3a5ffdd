"""Generate the golden vectors in tests/golden/ from the reference's own code.

Run in a container that holds the reference source tree:

    python tests/golden/make_golden.py [--ref-src /path/to/reference/src]

It builds oracle/_ref/ (a C ABI over the reference's headers, FP64 via a
force-included configuration and the default FP32) with oracle/Makefile, then
calls the reference's pair sweeps, compute_bonded, verlet_langevin,
the fused Nose-Hoover functors, compute_temperature, morton_encode and
init_rbc on seeded inputs, and writes the inputs and the reference's outputs
to small .npz fixtures.  The tests replay these inputs through the oracle and
the GPU library; nothing at test time needs the reference tree.
"""
from __future__ import annotations

import argparse
import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as orc  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def lattice(nx, ny, spacing=1.1, jitter=0.05, tilt=0.05, kT=1.0, seed=1):
    """Flat square lattice of lipids (the plain small workload's geometry)."""
    rng = np.random.default_rng(seed)
    ix, iy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    x = np.stack([ix.ravel() * spacing, iy.ravel() * spacing, np.zeros(nx * ny)], 1)
    x += rng.normal(0, jitter, x.shape)
    n = len(x)
    ang = rng.normal(0, tilt, n)
    phi = rng.uniform(0, 2 * np.pi, n)
    axis = np.stack([np.cos(phi), np.sin(phi), np.zeros(n)], 1)
    # rotate +z about an in-plane axis by ang: n = (sin(a) * (axis x z), cos(a))
    axz = np.cross(axis, np.array([0.0, 0.0, 1.0]))
    nrm = np.sin(ang)[:, None] * axz + np.cos(ang)[:, None] * np.array([0.0, 0.0, 1.0])
    v = rng.normal(0, np.sqrt(kT), (n, 3))
    o = rng.normal(0, 0.1, (n, 3))
    return x, nrm, v, o, np.zeros(n, np.int32), np.arange(1, n + 1, dtype=np.int32)


def icosahedron():
    t = (1 + 5 ** 0.5) / 2
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], float)
    v /= np.linalg.norm(v, axis=1)[:, None]
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]])
    # counter-clockwise seen from outside, the convention of the shipped mesh
    c = v[f].mean(1)
    nn = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    flip = np.sum(nn * c, 1) < 0
    f[flip] = f[flip][:, ::-1]
    e = set()
    for a, b, cc in f:
        for p, q in ((a, b), (b, cc), (cc, a)):
            e.add((min(p, q), max(p, q)))
    return v, np.array(sorted(e)), f


def whole_cell(prefix):
    v, e, f = icosahedron()
    np.savetxt(prefix + ".vert.txt", v, fmt="%.9f", delimiter="\t")
    np.savetxt(prefix + ".bond.txt", e, fmt="%d", delimiter="\t")
    np.savetxt(prefix + ".face.txt", f, fmt="%d", delimiter="\t")
    R = orc.ref("f64")
    cap, bcap = 200000, 200000
    x = np.zeros((cap, 3))
    nrm = np.zeros((cap, 3))
    ty = np.zeros(cap, np.int32)
    tg = np.zeros(cap, np.int32)
    b3 = np.zeros((bcap, 3), np.int32)
    nb = C.c_int64()
    area = C.c_double()
    n = R.ref_init_rbc(prefix.encode(), cap, x.ctypes.data, nrm.ctypes.data, ty.ctypes.data, tg.ctypes.data, bcap,
                       b3.ctypes.data, C.byref(nb), C.byref(area))
    assert n > 0
    return x[:n].copy(), nrm[:n].copy(), ty[:n].copy(), tg[:n].copy(), b3[:nb.value].copy(), area.value


def ref_forces(prec, x, nrm, ty, tg, bonds):
    R = orc.ref(prec)
    n = len(x)
    f = np.zeros((n, 3))
    t = np.zeros((n, 3))
    b = np.ascontiguousarray(bonds, np.int32)
    R.ref_forces(n, x.ctypes.data, nrm.ctypes.data, ty.ctypes.data, tg.ctypes.data, len(b),
                 b.ctypes.data if len(b) else None, f.ctypes.data, t.ctypes.data)
    return f, t


def ref_langevin(prec, x, nrm, v, o, ty, tg, bonds, dt, kBT, eta, nsteps):
    R = orc.ref(prec)
    x, nrm, v, o = (np.ascontiguousarray(a, np.float64).copy() for a in (x, nrm, v, o))
    b = np.ascontiguousarray(bonds, np.int32)
    R.ref_langevin(len(x), x.ctypes.data, nrm.ctypes.data, v.ctypes.data, o.ctypes.data, ty.ctypes.data,
                   tg.ctypes.data, len(b), b.ctypes.data if len(b) else None, dt, kBT, eta, nsteps)
    return x, nrm, v, o


def ref_nh(prec, x, nrm, v, o, ty, tg, bonds, dt, kBT, zeta, Q, nsteps):
    R = orc.ref(prec)
    x, nrm, v, o = (np.ascontiguousarray(a, np.float64).copy() for a in (x, nrm, v, o))
    b = np.ascontiguousarray(bonds, np.int32)
    z = C.c_double(zeta)
    R.ref_nh(len(x), x.ctypes.data, nrm.ctypes.data, v.ctypes.data, o.ctypes.data, ty.ctypes.data,
             tg.ctypes.data, len(b), b.ctypes.data if len(b) else None, dt, kBT, C.byref(z), Q, nsteps)
    return x, nrm, v, o, z.value


def ref_temperature(prec, x, nrm, v, ty, tg):
    R = orc.ref(prec)
    return R.ref_temperature(len(x), x.ctypes.data, nrm.ctypes.data, v.ctypes.data, ty.ctypes.data, tg.ctypes.data)


def lattice_config1():
    """The plain small workload: 32,768 lipids, row-major on a 182-column
    square lattice of spacing 1.1 (180 full rows and 8 sites), jitter 0.05,
    normals tilted 0.05 rad, Maxwell-Boltzmann velocities at kT = 1 -- the
    library's own generator (orbc_gen_lattice, seed 1), built by the oracle's
    Makefile.  The inputs are rounded to float32 so the fixture stays small
    (exact values in float64 for the reference).  Forces and torques by the
    reference's FP64 code at step 0, its FP32 forces, and 100 noise-free
    Langevin steps (kT = 0, eta = 0.01) in FP64, of which every fourth
    particle's final state is kept."""
    from openrbc_gb300 import workloads
    w = workloads.lattice(n=32768, ncol=182, spacing=1.1, jitter=0.05, tilt=0.05, kT=1.0, seed=1,
                          lib=orc.workloads_lib())
    x, nrm, v, o = (np.asarray(w[k], np.float32).astype(np.float64) for k in ("x", "n", "v", "o"))
    ty, tg = w["type"], w["tag"]
    nob = np.zeros((0, 3), np.int32)
    f64, t64 = ref_forces("f64", x, nrm, ty, tg, nob)
    f32, t32 = ref_forces("f32", x, nrm, ty, tg, nob)
    T = ref_temperature("f64", x, nrm, v, ty, tg)
    lx, ln, lv, lo = ref_langevin("f64", x, nrm, v, o, ty, tg, nob, 0.01, 0.0, 0.01, 100)
    keep = np.arange(0, len(x), 4)
    np.savez_compressed(os.path.join(OUT, "lattice_32768.npz"), x=x.astype(np.float32), nrm=nrm.astype(np.float32),
                        v=v.astype(np.float32), o=o.astype(np.float32), type=ty, tag=tg, f64=f64, t64=t64,
                        f32=f32.astype(np.float32), t32=t32.astype(np.float32), temperature=T,
                        lang_keep=keep.astype(np.int32), lang_x=lx[keep], lang_n=ln[keep], lang_v=lv[keep],
                        lang_o=lo[keep], lang_steps=100, lang_dt=0.01, lang_eta=0.01)
    print("lattice_32768:", len(x), "particles; |f|max", np.abs(f64).max())


def example_large_patch(ref_src, r_in=70.0, margin=6.0, seed=11):
    """The reference's own whole cell: init_rbc on example-large/rbc.{vert,
    bond,face}.txt (3.2M particles, 19-bead harmonic spectrin) by the
    reference's FP64 code.  A patch is cut around a seeded lipid: every
    particle within r_in + margin of it, with the bonds whose two ends are in
    the patch.  The margin exceeds every interaction range (largest 3.82, the
    protein-lipid WCA cut), so the forces on the particles within r_in whose
    bond partners are all in the patch (`check`) equal their forces in the
    whole cell; those are the reference's FP64 forces and torques on the
    patch."""
    prefix = os.path.join(os.path.dirname(os.path.abspath(ref_src)), "example-large", "rbc")
    R = orc.ref("f64")
    cap, bcap = 4_000_000, 1_000_000
    x = np.zeros((cap, 3))
    nrm = np.zeros((cap, 3))
    ty = np.zeros(cap, np.int32)
    tg = np.zeros(cap, np.int32)
    b3 = np.zeros((bcap, 3), np.int32)
    nb = C.c_int64()
    area = C.c_double()
    n = R.ref_init_rbc(prefix.encode(), cap, x.ctypes.data, nrm.ctypes.data, ty.ctypes.data, tg.ctypes.data, bcap,
                       b3.ctypes.data, C.byref(nb), C.byref(area))
    assert n > 0
    x, nrm, ty, tg, b3 = x[:n], nrm[:n], ty[:n], tg[:n], b3[:nb.value]
    rng = np.random.default_rng(seed)
    lip = np.flatnonzero(ty == 0)
    c = x[lip[rng.integers(len(lip))]]
    d = np.linalg.norm(x - c, axis=1)
    sel = np.flatnonzero(d < r_in + margin)
    inpatch = np.zeros(n, bool)
    inpatch[sel] = True
    idx_of_tag = np.full(int(tg.max()) + 1, -1, np.int64)
    idx_of_tag[tg] = np.arange(n)
    bi, bj = idx_of_tag[b3[:, 1]], idx_of_tag[b3[:, 2]]
    both = inpatch[bi] & inpatch[bj]
    one = inpatch[bi] ^ inpatch[bj]
    broken = np.zeros(n, bool)
    broken[bi[one]] = True
    broken[bj[one]] = True
    check = (d[sel] < r_in) & ~broken[sel]
    px, pn, pty, ptg, pb = x[sel], nrm[sel], ty[sel], tg[sel], b3[both]
    f64, t64 = ref_forces("f64", px, pn, pty, ptg, pb)
    np.savez_compressed(os.path.join(OUT, "example_large_patch.npz"), x=px, nrm=pn, type=pty, tag=ptg, bonds=pb,
                        check=check, f64=f64, t64=t64, cell_particles=n, cell_bonds=nb.value, mesh_area=area.value,
                        centre=c, r_in=r_in, margin=margin)
    print("example_large_patch:", len(sel), "particles of", n, "; checked", int(check.sum()), "; types",
          np.bincount(pty, minlength=6), "; bonds", len(pb))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", default="/root/reference/src", help="the reference's src/ directory")
    ap.add_argument("--only", default="", help="comma-separated fixture names to (re)make: lattice_576, cell_ico12, "
                                               "morton, frames, lattice_32768, example_large_patch")
    args = ap.parse_args()
    orc.build(args.ref_src)
    assert orc.ref_available("f64") and orc.ref_available("f32"), "reference harness did not build"
    assert orc.ref("f64").ref_real_bytes() == 8 and orc.ref("f32").ref_real_bytes() == 4
    only = set(filter(None, args.only.split(",")))
    if only:
        if "lattice_32768" in only:
            lattice_config1()
        if "example_large_patch" in only:
            example_large_patch(args.ref_src)
        return

    # ---- plain lipid lattice ------------------------------------------------
    x, nrm, v, o, ty, tg = lattice(24, 24)
    nob = np.zeros((0, 3), np.int32)
    f64, t64 = ref_forces("f64", x, nrm, ty, tg, nob)
    f32, t32 = ref_forces("f32", x, nrm, ty, tg, nob)
    lx, ln, lv, lo = ref_langevin("f64", x, nrm, v, o, ty, tg, nob, 0.01, 0.0, 0.01, 100)
    nx_, nn_, nv_, no_, nz = ref_nh("f64", x, nrm, v, o, ty, tg, nob, 0.01, 1.0, 0.0, 0.0, 20)
    T = ref_temperature("f64", x, nrm, v, ty, tg)
    np.savez_compressed(os.path.join(OUT, "lattice_576.npz"), x=x, nrm=nrm, v=v, o=o, type=ty, tag=tg,
                        f64=f64, t64=t64, f32=f32, t32=t32, temperature=T,
                        lang_x=lx, lang_n=ln, lang_v=lv, lang_o=lo, lang_steps=100, lang_dt=0.01, lang_eta=0.01,
                        nh_x=nx_, nh_n=nn_, nh_v=nv_, nh_o=no_, nh_zeta=nz, nh_steps=20, nh_dt=0.01, nh_kBT=1.0)
    print("lattice_576:", len(x), "particles; |f|max", np.abs(f64).max())

    # ---- whole cell on a 12-vertex mesh (all protein types, all bond types) --
    os.makedirs(orc.REF_DIR, exist_ok=True)
    x, nrm, ty, tg, bonds, area = whole_cell(os.path.join(orc.REF_DIR, "ico12"))
    rng = np.random.default_rng(7)
    m = np.array([1, 4, 4, 1, 10, 10], float)[ty]
    v = rng.normal(0, 1, (len(x), 3)) * np.sqrt(0.22 / m)[:, None]
    o = rng.normal(0, 0.05, (len(x), 3))
    f64, t64 = ref_forces("f64", x, nrm, ty, tg, bonds)
    f32, t32 = ref_forces("f32", x, nrm, ty, tg, bonds)
    lx, ln, lv, lo = ref_langevin("f64", x, nrm, v, o, ty, tg, bonds, 0.01, 0.0, 0.01, 20)
    nx_, nn_, nv_, no_, nz = ref_nh("f64", x, nrm, v, o, ty, tg, bonds, 0.01, 0.22, 0.0, 0.0, 10)
    T = ref_temperature("f64", x, nrm, v, ty, tg)
    np.savez_compressed(os.path.join(OUT, "cell_ico12.npz"), x=x, nrm=nrm, v=v, o=o, type=ty, tag=tg, bonds=bonds,
                        mesh_area=area, f64=f64, t64=t64, f32=f32, t32=t32, temperature=T,
                        lang_x=lx, lang_n=ln, lang_v=lv, lang_o=lo, lang_steps=20, lang_dt=0.01, lang_eta=0.01,
                        nh_x=nx_, nh_n=nn_, nh_v=nv_, nh_o=no_, nh_zeta=nz, nh_steps=10, nh_dt=0.01, nh_kBT=0.22)
    print("cell_ico12:", len(x), "particles,", len(bonds), "bonds; types", np.bincount(ty))

    # ---- Morton keys -----------------------------------------------------------
    rng = np.random.default_rng(3)
    p = rng.uniform(-1000, 1000, (4000, 3))
    edge = np.array([[-1000, -1000, -1000], [-488.5, -488.0, -487.5], [-488.01, 0, 0], [0, 0, 0],
                     [999.99, 999.99, 999.99], [-1000, 0, 1000], [-500.25, 12.75, -999.5]], float)
    p = np.concatenate([p, edge, rng.uniform(-1000, -480, (500, 3))])
    k64 = np.zeros(len(p), np.uint32)
    orc.ref("f64").ref_morton_encode(len(p), np.ascontiguousarray(p).ctypes.data, k64.ctypes.data)
    p32 = p.astype(np.float32).astype(np.float64)
    k32 = np.zeros(len(p), np.uint32)
    orc.ref("f32").ref_morton_encode(len(p), np.ascontiguousarray(p32).ctypes.data, k32.ctypes.data)
    np.savez_compressed(os.path.join(OUT, "morton.npz"), p=p, keys64=k64, p32=p32, keys32=k32)
    print("morton:", len(p), "points")

    # ---- trajectory frames (src/trajectory.h:61-105) ---------------------------
    # 48 lipids and 16 proteins interleaved; lipid tags are the reference's
    # implicit 1, 2, ... in input order, protein tags 1000 + k.
    g = np.load(os.path.join(OUT, "cell_ico12.npz"))
    lip = np.flatnonzero(g["type"] == 0)[:48]
    pro = np.flatnonzero(g["type"] != 0)[:16]
    sel = np.sort(np.concatenate([lip, pro]))
    fx, fn, fv = (np.ascontiguousarray(g[k][sel]) for k in ("x", "nrm", "v"))
    fty = np.ascontiguousarray(g["type"][sel]).astype(np.int32)
    ftg = np.zeros(len(sel), np.int32)
    ftg[fty == 0] = np.arange(1, int((fty == 0).sum()) + 1)
    ftg[fty != 0] = 1000 + np.arange(int((fty != 0).sum()))
    ff = np.random.default_rng(7).normal(0, 3.0, fx.shape)
    faff = np.random.default_rng(8).integers(0, 500, len(sel)).astype(np.int32)
    frames = {}
    for prec, fields, nstep in (("f32", 31, 120), ("f64", 31, 120), ("f32", 7, 0)):
        R = orc.ref(prec)
        vp = C.c_void_p
        R.ref_save_frame.restype = C.c_int64
        R.ref_save_frame.argtypes = [C.c_int64, vp, vp, vp, vp, vp, vp, vp, C.c_int, C.c_int, vp, C.c_int64]
        args = [C.c_int64(len(sel)), fx.ctypes.data, fn.ctypes.data, fv.ctypes.data, ff.ctypes.data,
                fty.ctypes.data, ftg.ctypes.data, faff.ctypes.data, C.c_int(nstep), C.c_int(fields)]
        size = R.ref_save_frame(*args, None, C.c_int64(0))
        buf = C.create_string_buffer(size)
        R.ref_save_frame(*args, buf, C.c_int64(size))
        frames[f"frame_{prec}_{fields}_{nstep}"] = np.frombuffer(buf.raw[:size], np.uint8)
    np.savez_compressed(os.path.join(OUT, "frames.npz"), x=fx, nrm=fn, v=fv, f=ff, type=fty, tag=ftg, affil=faff,
                        **frames)
    print("frames:", {k: len(v) for k, v in frames.items()})

    lattice_config1()
    example_large_patch(args.ref_src)


if __name__ == "__main__":
    main()
