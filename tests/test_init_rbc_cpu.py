"""Whole-cell initialiser, host part and checker (no GPU): the protein network
of orbc_init_rbc_network against the golden cell that the reference's own
init_rbc built from the same mesh (src/init_rbc.h:29-305), the lipid count
of every face, and the oracle's restatement of the lipid placement."""
import numpy as np

from conftest import geodesic_mesh, load_golden


def _network(freq=1, seed=0):
    from openrbc_gb300 import workloads
    v, e, f = geodesic_mesh(freq)
    return workloads.init_rbc_network(v, e, f, rho=1.05, seed=seed)


def test_network_matches_the_reference_init_rbc():
    g = load_golden("cell_ico12.npz")
    net = _network()
    npr = len(net["x"])
    assert npr == 624 and net["n_lipid"] == len(g["x"]) - npr == 2920
    assert np.array_equal(net["type"], g["type"][:npr])
    assert np.array_equal(net["tag"], g["tag"][:npr])
    assert np.array_equal(net["bonds"], g["bonds"])
    spectrin = net["type"] == 5
    # glycophorin, actin, band-III: same positions and normals, bit for bit
    assert np.array_equal(net["x"][~spectrin], g["x"][:npr][~spectrin])
    assert np.array_equal(net["n"], g["nrm"][:npr])          # spectrin normals: the noise-free bead position
    # spectrin beads: the same chain points, each coordinate displaced by its own noise in [-0.05, 0.05)
    assert np.abs(net["x"][spectrin] - g["x"][:npr][spectrin]).max() <= 0.1


def test_lipid_counts_per_face_match_the_reference():
    """The reference lays the lipids out face by face: with the same counts,
    the golden lipids of face f lie on face f's triangle."""
    g = load_golden("cell_ico12.npz")
    net = _network()
    npr = len(net["x"])
    lip = g["x"][npr:]
    base = np.concatenate([[0], np.cumsum(net["face_nl"])])
    for k, (a, b, c) in enumerate(net["face"]):
        p = lip[base[k]:base[k + 1]]
        va, vb, vc = net["vert"][a], net["vert"][b], net["vert"][c]
        nrm = net["face_normal"][k]
        assert np.abs((p - vb) @ nrm).max() < 1e-9
        # barycentric coordinates inside the triangle
        T = np.stack([va - vc, vb - vc], 1)
        lam, *_ = np.linalg.lstsq(T, (p - vc).T, rcond=None)
        assert lam.min() > -1e-9 and (lam.sum(0)).max() < 1 + 1e-9
        assert np.allclose(g["nrm"][npr:][base[k]:base[k + 1]], nrm, atol=1e-12)


def test_oracle_placement_keeps_the_exclusions():
    from oracle import oracle as orc
    for freq in (1, 2):
        net = _network(freq, seed=3)
        x, n = orc.place_lipids(net, seed=11)
        base = np.concatenate([[0], np.cumsum(net["face_nl"])])
        assert len(x) == net["n_lipid"]
        d = np.sqrt(((x[:, None, :] - net["x"][None, :, :]) ** 2).sum(2))
        assert d.min() >= 1.685
        for k, tri in enumerate(net["face"]):
            p = x[base[k]:base[k + 1]]
            if len(p) > 1:
                dd = np.sqrt(((p[:, None] - p[None]) ** 2).sum(2)) + 9 * np.eye(len(p))
                assert dd.min() >= 0.55
            assert np.linalg.norm(p - net["vert"][tri[0]], axis=1).min() >= 1.685
            assert np.array_equal(n[base[k]:base[k + 1]], np.tile(net["face_normal"][k], (len(p), 1)))
