"""Many-domain batch (include/aeros_batch.h) on the GPU.

The batch has no reference counterpart; its contract is that it changes no
result: every member's populations and fields are bitwise those of the same
domain stepped alone through aeros_lbm_step, whatever the other members, the
tuning or the time the member joined.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SMALL = ((32, 16, 16), (40, 24, 24), (24, 20, 16), (48, 16, 24))


@pytest.fixture(scope="module")
def mods():
    from aeros_gb300 import batch, capi, geometry, solver
    return batch, capi, geometry, solver


def domain(mods, i, storage="fp16", level=2):
    _, _, geometry, solver = mods
    p, mask, _ = geometry.batch_domain(i, storage=storage, level=level, sizes=SMALL)
    return solver.Solver(p, mask), p, mask


def state(s):
    f = s.fields()
    return s.populations(), {k: f[k] for k in ("rho", "ux", "uy", "uz")}, s.stats()


def assert_same(a, b, stats_bitwise=True):
    fa, va, sa = a
    fb, vb, sb = b
    assert np.array_equal(fa, fb)
    for k in va:
        assert np.array_equal(va[k], vb[k]), k
    assert sa["step"] == sb["step"]
    if stats_bitwise:
        assert sa["sum_rho"] == sb["sum_rho"] and sa["sum_kinetic"] == sb["sum_kinetic"]
        assert sa["max_velocity_lb"] == sb["max_velocity_lb"]


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_batch_members_equal_lone_domains(mods, storage):
    """Populations and fields after 40 batch steps are bitwise the lone
    aeros_lbm_step result; statistics agree to rounding (other sum order)."""
    Batch = mods[0].Batch
    with Batch(storage) as b:
        members = [domain(mods, i, storage)[0] for i in range(4)]
        for s in members:
            b.add(s)
        b.set_tuning(chunk_steps=10)
        b.step(40)
        got = [state(s) for s in members]
        assert b.last_launch_count() == 80   # shell + interior launch per step
    for i, g in enumerate(got):
        s, _, _ = domain(mods, i, storage)
        s.step(40)
        ref = state(s)
        assert_same(g, ref, stats_bitwise=False)
        assert abs(g[2]["sum_rho"] - ref[2]["sum_rho"]) <= 1e-9 * ref[2]["sum_rho"]
        assert abs(g[2]["avg_kinetic"] - ref[2]["avg_kinetic"]) <= 1e-5 * ref[2]["avg_kinetic"]


def test_alone_and_in_mix_identical(mods):
    """A member alone in a batch and in a mix of four: same bits, statistics
    included (per-tile partials summed in tile order)."""
    Batch = mods[0].Batch
    with Batch("fp16") as b:
        s, _, _ = domain(mods, 1)
        b.add(s)
        b.step(30)
        alone = state(s)
        b.remove(s)
    with Batch("fp16") as b:
        ms = [domain(mods, i)[0] for i in range(4)]
        for m in ms:
            b.add(m)
        b.step(30)
        mixed = state(ms[1])
    assert_same(alone, mixed)


def test_tuning_changes_no_result(mods):
    Batch = mods[0].Batch
    outs = []
    for tune in (dict(blocks_per_sm=1, tiles_per_item=1, shell_tiles_per_item=1, chunk_steps=4),
                 dict(blocks_per_sm=0, tiles_per_item=4, shell_tiles_per_item=8, chunk_steps=12)):
        with Batch("fp16") as b:
            ms = [domain(mods, i)[0] for i in range(3)]
            for m in ms:
                b.add(m)
            b.set_tuning(**tune)
            b.step(24)
            outs.append([state(m) for m in ms])
    for a, c in zip(*outs):
        assert_same(a, c)


def test_autotune_picks_a_shape_and_keeps_results(mods):
    Batch = mods[0].Batch
    with Batch("fp16") as b:
        ms = [domain(mods, i)[0] for i in range(3)]
        for m in ms:
            b.add(m)
        best = b.autotune(trial_steps=4)
        assert best["tiles_per_item"] in (1, 2, 4) and best["blocks_per_sm"] >= 1
        steps = ms[0].stats()["step"]
        b.step(10)
        got = [state(m) for m in ms]
    for i, g in enumerate(got):
        s, _, _ = domain(mods, i)
        s.step(steps + 10)
        assert_same(g, state(s), stats_bitwise=False)


def test_member_joining_later(mods):
    """A domain added after the others have run starts from its own step 0."""
    Batch = mods[0].Batch
    with Batch("fp16") as b:
        a, _, _ = domain(mods, 0)
        b.add(a)
        b.step(20)
        c, _, _ = domain(mods, 2)
        b.add(c)
        b.step(20)
        got_a, got_c = state(a), state(c)
    ra, _, _ = domain(mods, 0)
    ra.step(40)
    rc, _, _ = domain(mods, 2)
    rc.step(20)
    assert_same(got_a, state(ra), stats_bitwise=False)
    assert_same(got_c, state(rc), stats_bitwise=False)


def test_diverged_member_is_reset_alone(mods):
    """NaN populations in one member trip its divergence guard; it is
    re-equilibrated and the other members are untouched."""
    Batch = mods[0].Batch
    with Batch("fp32") as b:
        ms = [domain(mods, i, "fp32")[0] for i in range(3)]
        for m in ms:
            b.add(m)
        b.step(10)
        f = ms[1].populations()
        f[:, :] = np.nan
        ms[1].write_populations(f)
        b.step(10)
        assert ms[1].stats()["diverged"] == 1
        assert ms[0].stats()["diverged"] == 0
        got0 = state(ms[0])
        b.step(10)
        assert np.isfinite(ms[1].fields()["ux"]).all()
    r0, _, _ = domain(mods, 0, "fp32")
    r0.step(20)
    assert_same(got0, state(r0), stats_bitwise=False)


def test_batch_rejects_bad_calls(mods):
    batch, capi, _, _ = mods
    with batch.Batch("fp16") as b:
        s, _, _ = domain(mods, 0)
        b.add(s)
        with pytest.raises(capi.AerosError):
            b.add(s)                       # already a member
        with pytest.raises(capi.AerosError):
            b.step(3)                      # odd step count
        with pytest.raises(capi.AerosError):
            capi.check(capi.lib().aeros_lbm_destroy(s.h), "destroy")   # still a member
        t32, _, _ = domain(mods, 1, "fp32")
        with pytest.raises(capi.AerosError):
            b.add(t32)                     # other storage
        lone, _, _ = domain(mods, 2)
        lone.step(1)
        with pytest.raises(capi.AerosError):
            b.add(lone)                    # odd AA parity
        b.remove(s)
        assert b.size() == (0, 0)
