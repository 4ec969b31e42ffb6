"""Continuous-batching MD serving (cg_md_serve): results alone and in the mix for the
FP32 contraction form on the 4-body serving basis, and the device-memory admission.

Tolerances: a request's final positions after its steps are the same alone and in
a mixed batch within 1e-8 A (FP32 per-cluster forces are computed the same way in
both; the FP64 force sums are reordered by atomics).
"""
import importlib
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
MASSES = np.array([12.011, 1.0079, 14.007, 15.9994])


def _requests(cg, tmp_path, sizes, order, seed, nsteps, spacing):
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    fm = synth.make_workload("chno-4b", str(tmp_path), nframes=len(sizes), seed=seed, order=order,
                             sizes=list(sizes), triclinic=False, density=0.1, labels=False)
    model = cg.Model(fm)
    nat, types, xyz, cell = synth.frames_arrays(os.path.join(str(tmp_path), "traj.xyzf"), len(sizes),
                                                ["C", "H", "N", "O"])[:4]
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(model.ncols) * 1e-4
    ofs = np.concatenate([[0], np.cumsum(nat)])
    reqs = []
    for k in range(len(sizes)):
        a, b = ofs[k], ofs[k + 1]
        v = rng.standard_normal((b - a, 3)) * np.sqrt(0.0019872067 * 300.0 / MASSES[types[a:b]])[:, None]
        reqs.append(dict(types=types[a:b], xyz=xyz[a:b], cell=cell[k], v=v, nsteps=nsteps, arrival=spacing * k))
    return model, x, reqs


def test_serving_fp32_same_alone_and_in_the_mix(cg, tmp_path):
    """The serving basis (2B 16 / 3B 8 / 4B 4 at 5.0 / 4.0 / 3.5 A, 4 species) with
    requests of about 1024 atoms arriving while others run, FP32 contraction form."""
    model, x, reqs = _requests(cg, tmp_path, [1024, 700, 1100, 900], (16, 8, 4), 123, 10, 0.002)
    sess = cg.Session(model, 0)
    sess.md_setup(x, precision=cg.CG_FP32)
    mix, res, step_ms, nb = sess.md_serve(reqs, MASSES, dt_fs=0.2, max_batch_atoms=4096, max_batch_frames=4)
    alone, res1, _, nb1 = sess.md_serve(reqs, MASSES, dt_fs=0.2, max_batch_frames=1)
    assert nb1 == 10 * len(reqs) and nb < nb1
    worst = max(float(np.abs(m - a).max()) for m, a in zip(mix, alone))
    moved = max(float(np.abs(m - q["xyz"]).max()) for m, q in zip(mix, reqs))
    print(f"\nFP32 serving: {nb} batched steps vs {nb1} alone; largest |mix - alone| = {worst:.3e} A "
          f"(atoms moved up to {moved:.3e} A)", flush=True)
    assert moved > 1e-4
    assert worst <= 1e-8


def test_serving_budget_defers_a_request(cg, tmp_path):
    """Two requests arriving together under a budget with room for one: the second is
    admitted only after the first has finished, and both give the results they give
    under an ample budget."""
    model, x, reqs = _requests(cg, tmp_path, [120, 110], (8, 4, 3), 5, 8, 0.0)
    sess = cg.Session(model, 0)
    sess.md_setup(x)
    ample, res0, _, _ = sess.md_serve(reqs, MASSES, dt_fs=0.2, max_batch_atoms=512, max_batch_frames=4)
    assert res0["admitted"][1] < res0["finished"][0]          # both ran together
    arena, per_atom = sess.md_serve_memory(512, 4)             # measured by the run above
    assert arena > 0 and per_atom > 0
    budget = arena + per_atom * 180                            # room for one request, not two
    tight, res, _, _ = sess.md_serve(reqs, MASSES, dt_fs=0.2, hbm_budget=budget, max_batch_atoms=512,
                                     max_batch_frames=4)
    assert res["admitted"][1] >= res["finished"][0]
    assert np.all(res["reserved_bytes"] > 0)
    for a, t in zip(ample, tight):
        assert np.abs(a - t).max() <= 1e-9


def test_serving_refuses_budgets_it_cannot_meet(cg, tmp_path):
    """A budget below the arenas, or one that no single request fits, is an error
    (status 1), not an endless wait."""
    model, x, reqs = _requests(cg, tmp_path, [120, 110], (8, 4, 3), 6, 4, 0.0)
    sess = cg.Session(model, 0)
    sess.md_setup(x)
    arena, per_atom = sess.md_serve_memory(512, 4)
    for budget in (0.5 * arena, arena + 10.0 * per_atom):
        with pytest.raises(cg.ChimesError) as e:
            sess.md_serve(reqs, MASSES, dt_fs=0.2, hbm_budget=budget, max_batch_atoms=512, max_batch_frames=4)
        assert e.value.code == 1


def test_live_server_same_as_alone(cg, tmp_path):
    """cg_md_server_*: a client thread submits requests at intervals while earlier
    ones are on the GPU; every result equals the same request run alone through
    cg_md_serve (FP32 form, 1e-8 A), requests overlap in batched steps, a request too
    large for the batch is refused at submission, and poll reports unfinished tickets
    as pending."""
    import threading
    import time
    model, x, reqs = _requests(cg, tmp_path, [1024, 700, 1100, 900, 300], (16, 8, 4), 321, 12, 0.0)
    sess = cg.Session(model, 0)
    sess.md_setup(x, precision=cg.CG_FP32)
    alone, _, _, _ = sess.md_serve(reqs, MASSES, dt_fs=0.2, max_batch_frames=1)
    srv = sess.md_server(MASSES, dt_fs=0.2, max_batch_atoms=4096, max_batch_frames=4)
    tickets = []
    with pytest.raises(RuntimeError):
        srv.submit(np.zeros(5000, dtype=np.int32), np.zeros((5000, 3)), reqs[0]["cell"], np.zeros((5000, 3)), 1)

    def client():
        for q in reqs:
            tickets.append(srv.submit(q["types"], q["xyz"], q["cell"], q["v"], q["nsteps"]))
            time.sleep(0.002)

    th = threading.Thread(target=client)
    th.start()
    th.join()
    pending_seen = any(srv.poll(t) is None for t in tickets)
    outs = [srv.poll(t, wait=True) for t in tickets]
    nb = srv.stop()
    worst = max(float(np.abs(o[0] - a).max()) for o, a in zip(outs, alone))
    overlap = sum(1 for i in range(len(outs)) for j in range(i + 1, len(outs))
                  if outs[i][1]["admitted"] < outs[j][1]["finished"] and outs[j][1]["admitted"] < outs[i][1]["finished"])
    print(f"\nlive server: {nb} batched steps for {len(reqs)} requests of 12 steps; overlapping pairs {overlap}; "
          f"largest |server - alone| = {worst:.3e} A; pending seen {pending_seen}", flush=True)
    assert worst <= 1e-8
    assert overlap > 0 and nb < 12 * len(reqs)
    assert all(o[1]["finished"] >= o[1]["admitted"] for o in outs)
