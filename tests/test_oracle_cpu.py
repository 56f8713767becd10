"""The CPU oracle against the reference's own golden vectors and known answers.

The reference ships no tests or fixtures; its python/lct.py functions are the
only code of the reference that runs on a CPU, so the LCT fixtures in
tests/golden/ (made by importing lct.py) pin the LCT restatement.  The
backprojection/filter restatements are pinned here against hand-derived
known-answer cases and against pure-Python loops written straight from the
reference kernels; on the GPU the same oracle is pinned against the
reference's compiled kernels (tests/test_ref_parity_gpu.py).
"""
import math
from pathlib import Path

import numpy as np
import pytest

from oracle import cpu, numpy_ref
from tests.conftest import rel_l2

GOLDEN = Path(__file__).resolve().parent / "golden" / "lct_golden.npz"


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="module", autouse=True)
def _oracle_built(built):
    return built


# ------------------------------------------------------------------ LCT pins

@pytest.mark.parametrize("U,V", [(4, 8), (8, 16), (8, 32), (16, 16)])
def test_psf_matches_reference_lct_py(golden, U, V):
    psf = numpy_ref.define_psf(U, V, float(golden[f"psf_{U}_{V}_slope"]))
    np.testing.assert_array_equal(psf, golden[f"psf_{U}_{V}"])


@pytest.mark.parametrize("M", [8, 16, 32, 64])
def test_resampling_operator_matches_reference_lct_py(golden, M):
    mtx, mtxi = numpy_ref.resampling_operator(M)
    np.testing.assert_allclose(mtx.toarray(), golden[f"mtx_{M}"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(mtxi.toarray(), golden[f"mtxi_{M}"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("name", ["lct_a", "lct_b"])
def test_lct_matches_reference_lct_py(golden, name):
    width, bl, snr, diffuse = golden[f"{name}_params"]
    vol = numpy_ref.lct(golden[f"{name}_data"].astype(np.float64), width, bl, snr, bool(diffuse))
    assert rel_l2(vol, golden[f"{name}_vol"]) < 1e-12


def test_lct_grid_modes_differ_only_in_radiometry(golden):
    data = golden["lct_a_data"].astype(np.float64)
    a = numpy_ref.lct(data, 1.0, 0.03, grid="reference")
    b = numpy_ref.lct(data, 1.0, 0.03, grid="depth")
    assert a.shape == b.shape and not np.allclose(a, b)


@pytest.mark.parametrize("U,V,slope", [(4, 8, 0.3), (8, 16, 0.1), (16, 32, 0.05)])
def test_lct2_psf_centre_cancels_under_l2_normalisation(U, V, slope):
    """python/lct_2.py normalises the PSF by its column at (U, U) where lct.py
    uses (U - 1, U - 1); the L2 normalisation that follows removes any scalar,
    so both give the same PSF (which is why fbp_lct needs no option for it)."""
    a = numpy_ref.define_psf(U, V, slope)
    b = numpy_ref.define_psf(U, V, slope, center=U)
    np.testing.assert_allclose(a, b, rtol=1e-14, atol=1e-16)


def test_resampling_operator_rejects_non_power_of_two():
    with pytest.raises(ValueError):
        numpy_ref.resampling_operator(48)


# -------------------------------------------------------- filter_H restatement

def _direct_filter(h, step, wl_mean, border="zero"):
    """filter_H as the literal circular convolution of the padded series."""
    sigma, t6, n = numpy_ref.filter_h_params(h.shape[-1], step, wl_mean)
    K = numpy_ref.filter_h_kernel(n, float(np.float32(step)), float(np.float32(wl_mean)), sigma)
    T = h.shape[-1]
    pad = (n - T) // 2
    hp = np.zeros(n)
    hp[pad:pad + T] = h
    if border == "edge":
        hp[:pad] = h[0]
        hp[pad + T:] = h[-1]
    out = np.zeros(T)
    for t in range(T):
        tt = t + pad
        out[t] = n * sum(hp[u] * K[(tt - u) % n].real for u in range(n))
    return out


@pytest.mark.parametrize("border", ["zero", "edge"])
def test_filter_h_fft_equals_circular_correlation(border):
    rng = np.random.default_rng(0)
    h = rng.poisson(3.0, 40).astype(np.float64)
    step = 0.0048
    ref = _direct_filter(h, step, 10 * step, border)
    got = numpy_ref.filter_h(h[None], step, border=border)[0]
    np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-10)


def test_filter_h_padding_is_82_bins_for_default_wavelength():
    # wl_mean = 10 * deltaT gives t6sigma = 42 and nt_pad = nt + 82.
    _, t6, n = numpy_ref.filter_h_params(1024, 0.0048, 0.048)
    assert (t6, n) == (42, 1106)


# ------------------------------------------------------ backprojection oracle

def _info(L, T, step, vres, hmin, vs, discard=1, t0=0.0, S=None, laser_pos=(0.1, -0.4, 0.2),
          sensor_pos=(-0.2, -0.3, 0.1), system=0):
    o = cpu.OracleInfo()
    o.num_laser_targets = L
    o.num_sensor_targets = L if S is None else S
    o.num_time_bins = T
    o.time_step = step
    o.time_offset = t0
    o.discard_first_last_bounces = discard
    o.capture_system = system
    for k in range(3):
        o.voxel_res[k] = vres[k]
        o.hidden_min[k] = hmin[k]
        o.voxel_size[k] = vs[k]
        o.laser_position[k] = laser_pos[k]
        o.sensor_position[k] = sensor_pos[k]
    o.wall_normal[1] = -1.0
    return o


def _loop_confocal(o, cube_tmajor, lxyz):
    """Pure-Python restatement of backprojectConfocalVoxel
    (transient_reconstruction.cuh:93-136), FP64, cube[t*L + l]."""
    Vx, Vy, Vz = o.voxel_res
    L, T = o.num_laser_targets, o.num_time_bins
    vol = np.zeros((Vz, Vy, Vx))
    lp = np.array(o.laser_position[:], dtype=np.float64)
    sp = np.array(o.sensor_position[:], dtype=np.float64)
    for vz in range(Vz):
        for vy in range(Vy):
            for vx in range(Vx):
                p = np.array([o.hidden_min[0] + vx * o.voxel_size[0] + 0.5 * o.voxel_size[0],
                              o.hidden_min[1] + vz * o.voxel_size[1] + 0.5 * o.voxel_size[1],
                              o.hidden_min[2] + vy * o.voxel_size[2] + 0.5 * o.voxel_size[2]])
                for l in range(L):
                    q = lxyz[l].astype(np.float64)
                    dist = np.linalg.norm(p - q) * 2.0 - o.time_offset
                    if o.discard_first_last_bounces == 0:
                        dist += np.linalg.norm(q - lp) + np.linalg.norm(q - sp)
                    x = dist / o.time_step
                    if not (x > -1 and x < T):
                        continue
                    b = int(x)
                    I = cube_tmajor[b * L + l]
                    if I > np.float32(1e-5):
                        d2 = dist * dist
                        w = 1.0 / d2 if abs(d2) > 1e-5 else np.finfo(np.float32).max
                        vol[vz, vy, vx] += I * w
    return vol


@pytest.mark.parametrize("discard,t0", [(1, 0.0), (0, 0.0), (1, 0.05)])
def test_confocal_oracle_matches_python_loop(discard, t0):
    rng = np.random.default_rng(5)
    L, T = 9, 64
    lxyz = np.stack([rng.uniform(-1, 1, L), np.zeros(L), rng.uniform(-1, 1, L)], 1).astype(np.float32)
    o = _info(L, T, 0.05, (3, 4, 5), (-0.5, -1.2, -0.4), (0.3, 0.2, 0.25), discard, t0)
    cube = rng.uniform(0, 2, (T, L)).astype(np.float32)  # time-major
    cube[cube < 0.3] = 0
    want = _loop_confocal(o, cube.ravel(), lxyz)
    got_tm = cpu.confocal_voxel(o, cube, lxyz, layout=cpu.LAYOUT_TIME_MAJOR)
    got_ti = cpu.confocal_voxel(o, np.ascontiguousarray(cube.T), lxyz, layout=cpu.LAYOUT_TIME_INNER)
    np.testing.assert_allclose(got_tm, want, rtol=1e-12)
    np.testing.assert_array_equal(got_tm, got_ti)


def test_confocal_oracle_known_answer_single_pair():
    # One scan point at the origin, one voxel straight below at depth 0.5:
    # dist = 1.0 m, step 0.1 -> bin 10, weight 1/dist^2 = 1.
    o = _info(1, 32, 0.1, (1, 1, 1), (-0.05, -0.55, -0.05), (0.1, 0.1, 0.1))
    cube = np.zeros((1, 32), np.float32)
    cube[0, 10] = 3.0
    vol = cpu.confocal_voxel(o, cube, np.zeros((1, 3), np.float32))
    assert vol.shape == (1, 1, 1)
    assert vol[0, 0, 0] == pytest.approx(3.0, rel=1e-6)  # geometry is float32
    cube[0, 10] = 1e-6  # at or below EPS: skipped like the reference
    assert cpu.confocal_voxel(o, cube, np.zeros((1, 3), np.float32))[0, 0, 0] == 0.0


def _loop_scatter(o, cube_tmajor, lxyz):
    """Pure-Python restatement of the ACCUMULATE_VOXEL_SCATTERING build
    (transient_reconstruction.cuh:112-126), FP64, cube[t*L + l]."""
    Vx, Vy, Vz = o.voxel_res
    L, T = o.num_laser_targets, o.num_time_bins
    vol = np.zeros((Vz, Vy, Vx))
    lp = np.array(o.laser_position[:], dtype=np.float64)
    sp = np.array(o.sensor_position[:], dtype=np.float64)
    vs = np.array(o.voxel_size[:], dtype=np.float64)
    ext = 0.5 * float(np.sqrt(vs @ vs))
    step = o.time_step + float(np.float32(1e-5))
    for vz in range(Vz):
        for vy in range(Vy):
            for vx in range(Vx):
                p = np.array([o.hidden_min[0] + vx * vs[0] + 0.5 * vs[0], o.hidden_min[1] + vz * vs[1] + 0.5 * vs[1],
                              o.hidden_min[2] + vy * vs[2] + 0.5 * vs[2]])
                for l in range(L):
                    q = lxyz[l].astype(np.float64)
                    dist = np.linalg.norm(p - q) * 2.0 - o.time_offset
                    if o.discard_first_last_bounces == 0:
                        dist += np.linalg.norm(q - lp) + np.linalg.norm(q - sp)
                    d2 = dist * dist
                    w = 1.0 / d2 if abs(d2) > 1e-5 else np.finfo(np.float32).max
                    d = max(0.0, dist - ext)
                    while d < dist + ext:
                        x = d / o.time_step
                        if not (x > -1 and x < T):
                            break  # the reference's thread returns
                        I = cube_tmajor[int(x) * L + l]
                        if I > np.float32(1e-5):
                            vol[vz, vy, vx] += I * w
                        d += step
    return vol


@pytest.mark.parametrize("discard,t0", [(1, 0.0), (0, 0.0), (1, 0.05)])
def test_scatter_oracle_matches_python_loop(discard, t0):
    rng = np.random.default_rng(9)
    L, T = 9, 64
    lxyz = np.stack([rng.uniform(-1, 1, L), np.zeros(L), rng.uniform(-1, 1, L)], 1).astype(np.float32)
    o = _info(L, T, 0.05, (3, 4, 5), (-0.5, -1.2, -0.4), (0.3, 0.2, 0.25), discard, t0)
    cube = rng.uniform(0, 2, (T, L)).astype(np.float32)  # time-major
    cube[cube < 0.3] = 0
    want = _loop_scatter(o, cube.ravel(), lxyz)
    got_tm = cpu.confocal_scatter_voxel(o, cube, lxyz, layout=cpu.LAYOUT_TIME_MAJOR)
    got_ti = cpu.confocal_scatter_voxel(o, np.ascontiguousarray(cube.T), lxyz, layout=cpu.LAYOUT_TIME_INNER)
    np.testing.assert_allclose(got_tm, want, rtol=1e-12)
    np.testing.assert_array_equal(got_tm, got_ti)
    # Several bins per pair: the walk adds more than the single-bin form.
    assert got_tm.sum() > cpu.confocal_voxel(o, cube, lxyz, layout=cpu.LAYOUT_TIME_MAJOR).sum()


def test_scatter_oracle_known_answer_and_walk_end():
    # dist = 1.0 m, voxel diagonal sqrt(0.03) -> ext 0.0866; steps of 0.1 + 1e-5
    # from 0.9134 visit bins 9 and 10 (the next start, 1.1134, is past 1.0866).
    o = _info(1, 32, 0.1, (1, 1, 1), (-0.05, -0.55, -0.05), (0.1, 0.1, 0.1))
    cube = np.zeros((1, 32), np.float32)
    cube[0, 9], cube[0, 10], cube[0, 11] = 2.0, 3.0, 7.0
    lx = np.zeros((1, 3), np.float32)
    assert cpu.confocal_scatter_voxel(o, cube, lx)[0, 0, 0] == pytest.approx(5.0, rel=1e-6)
    # T = 10: bin 10 is outside the capture, the walk stops there.
    o.num_time_bins = 10
    assert cpu.confocal_scatter_voxel(o, np.ascontiguousarray(cube[:, :10]), lx)[0, 0, 0] == pytest.approx(2.0,
                                                                                                          rel=1e-6)


def test_scatter_float32_replay_agrees_with_fp64_walk():
    """numpy_ref.confocal_scatter_given_paths (the float32 replay of the walk
    from given FP32 paths, used with the GPU's paths in the GPU tests) against
    the FP64 oracle walk, with paths and constants rounded to float32 here:
    the known answer exactly, and a random case within the bin-edge flips."""
    o = _info(1, 32, 0.1, (1, 1, 1), (-0.05, -0.55, -0.05), (0.1, 0.1, 0.1))
    cube = np.zeros((1, 32), np.float32)
    cube[0, 9], cube[0, 10], cube[0, 11] = 2.0, 3.0, 7.0
    ext = float(np.float32(0.5 * math.sqrt(0.03)))
    got = numpy_ref.confocal_scatter_given_paths(cube, np.array([[1.0]], np.float32), float(np.float32(10.0)), ext, 0.1)
    assert got[0] == pytest.approx(5.0, rel=1e-6)
    # The walk stops at the first bin outside [0, T).
    got = numpy_ref.confocal_scatter_given_paths(np.ascontiguousarray(cube[:, :10]), np.array([[1.0]], np.float32),
                                                 float(np.float32(10.0)), ext, 0.1)
    assert got[0] == pytest.approx(2.0, rel=1e-6)

    rng = np.random.default_rng(19)
    L, T = 9, 64
    lxyz = np.stack([rng.uniform(-1, 1, L), np.zeros(L), rng.uniform(-1, 1, L)], 1).astype(np.float32)
    o = _info(L, T, 0.05, (3, 4, 5), (-0.5, -1.2, -0.4), (0.3, 0.2, 0.25))
    cube = rng.uniform(0, 2, (T, L)).astype(np.float32)
    cube[cube < 0.3] = 0
    want = cpu.confocal_scatter_voxel(o, np.ascontiguousarray(cube.T), lxyz).ravel()
    Vx, Vy, Vz = o.voxel_res
    vs = np.array(o.voxel_size[:], dtype=np.float64)
    paths = np.empty((Vx * Vy * Vz, L), np.float32)
    for v in range(Vx * Vy * Vz):
        vz, vy, vx = v // (Vx * Vy), (v // Vx) % Vy, v % Vx
        p = np.array(o.hidden_min[:]) + np.array([vx, vz, vy]) * vs + 0.5 * vs
        paths[v] = (2.0 * np.linalg.norm(lxyz.astype(np.float64) - p, axis=1)).astype(np.float32)
    got = numpy_ref.confocal_scatter_given_paths(np.ascontiguousarray(cube.T), paths,
                                                 float(np.float32(1.0 / o.time_step)),
                                                 float(np.float32(0.5 * math.sqrt(vs @ vs))), o.time_step)
    assert rel_l2(got, want) < 2e-2


def test_confocal_subset_matches_full():
    rng = np.random.default_rng(3)
    L, T = 16, 128
    lxyz = np.stack([rng.uniform(-1, 1, L), np.zeros(L), rng.uniform(-1, 1, L)], 1).astype(np.float32)
    o = _info(L, T, 0.03, (6, 5, 7), (-0.9, -1.5, -0.9), (0.3, 0.2, 0.35))
    cube = rng.poisson(0.5, (L, T)).astype(np.float32)
    full = cpu.confocal_voxel(o, cube, lxyz)
    idx = np.array([0, 7, 33, 100, 209], dtype=np.int64)
    np.testing.assert_allclose(cpu.confocal_voxel_subset(o, cube, lxyz, idx), full.ravel()[idx], rtol=1e-13)
    f32 = cpu.confocal_voxel_f32_subset(o, cube, lxyz, idx)
    np.testing.assert_allclose(f32, full.ravel()[idx], rtol=1e-4)
    # Given bins: the subset reads row i of its bins for voxel idx[i].
    V = 6 * 5 * 7
    bins = rng.integers(-3, T + 3, size=(V, L)).astype(np.int32)
    full_b = cpu.confocal_voxel(o, cube, lxyz, bins=bins)
    np.testing.assert_array_equal(cpu.confocal_voxel_subset(o, cube, lxyz, idx, bins=bins[idx]), full_b.ravel()[idx])


def test_exhaustive_oracle_matches_python_loop():
    rng = np.random.default_rng(9)
    L, S, T = 3, 4, 48
    lxyz = np.stack([rng.uniform(-1, 1, L), np.zeros(L), rng.uniform(-1, 1, L)], 1).astype(np.float32)
    sxyz = np.stack([rng.uniform(-1, 1, S), np.zeros(S), rng.uniform(-1, 1, S)], 1).astype(np.float32)
    o = _info(L, T, 0.06, (3, 2, 4), (-0.5, -1.2, -0.4), (0.3, 0.3, 0.25), discard=0, S=S, system=1)
    cube = rng.uniform(0, 2, (L, S, T)).astype(np.float32)
    got = cpu.exhaustive_voxel(o, cube, lxyz, sxyz)
    Vx, Vy, Vz = o.voxel_res
    want = np.zeros((Vz, Vy, Vx))
    lp = np.array(o.laser_position[:])
    sp = np.array(o.sensor_position[:])
    for vz in range(Vz):
        for vy in range(Vy):
            for vx in range(Vx):
                p = np.array([o.hidden_min[0] + (vx + 0.5) * o.voxel_size[0],
                              o.hidden_min[1] + (vz + 0.5) * o.voxel_size[1],
                              o.hidden_min[2] + (vy + 0.5) * o.voxel_size[2]])
                for l in range(L):
                    for s in range(S):
                        dist = (np.linalg.norm(p - lxyz[l]) + np.linalg.norm(p - sxyz[s])
                                + np.linalg.norm(lxyz[l] - lp) + np.linalg.norm(sxyz[s] - sp))
                        b = int(dist / o.time_step)
                        if 0 <= b < T and cube[l, s, b] > np.float32(1e-5):
                            want[vz, vy, vx] += cube[l, s, b] / dist ** 2
    np.testing.assert_allclose(got, want, rtol=1e-10)


def test_depth_oracles_are_unweighted_sums():
    rng = np.random.default_rng(2)
    L, T = 4, 256
    lxyz = np.stack([rng.uniform(-1, 1, L), np.zeros(L), rng.uniform(-1, 1, L)], 1).astype(np.float32)
    o = _info(L, T, 0.05, (1, 1, 1), (0, 0, 0), (1, 1, 1))
    cube = np.ones((L, T), np.float32)
    depths = np.array([0.3, 0.5, 0.7])
    act = cpu.depth_confocal(o, cube, lxyz, depths)
    # every pair lands inside T here, so each test point counts L ones.
    np.testing.assert_array_equal(act, np.full((L, 3), float(L)))
    o2 = _info(L, T, 0.05, (1, 1, 1), (0, 0, 0), (1, 1, 1), S=L, system=1)
    act2 = cpu.depth_exhaustive(o2, np.ones((L, L, T), np.float32), lxyz, lxyz, depths)
    np.testing.assert_array_equal(act2, np.full((L, 3), float(L * L)))


# ------------------------------------------------------------ filters & misc

def test_log_weights_sum_to_zero_and_are_symmetric():
    w = cpu.log_weights(5, 1.0).reshape(5, 5, 5)
    assert abs(float(w.astype(np.float64).sum())) < 1e-6
    np.testing.assert_array_equal(w, w[::-1, :, :])
    np.testing.assert_array_equal(w, np.transpose(w, (2, 1, 0)))
    assert w[2, 2, 2] == w.min()  # negative centre


def test_log_filter_of_constant_volume_is_zero_sum():
    w = cpu.log_weights(5, 1.0)
    out = cpu.log_filter(np.full((6, 7, 8), 2.0, np.float32), w, 5)
    assert np.abs(out).max() < 1e-5


def test_laplacian_known_answer():
    v = np.zeros((5, 5, 5), np.float32)
    v[2, 2, 2] = 1.0
    out = cpu.laplacian_filter(v, 3)
    assert out[2, 2, 2] == pytest.approx(26.0)
    assert out[1, 2, 2] == pytest.approx(-1.0)
    assert out[0, 0, 0] == 0.0


def test_normalize_known_answer():
    v = np.array([2.0, 4.0, 3.0])
    np.testing.assert_allclose(cpu.normalize(v), [0.0, 1.0, 0.5])
    # max == min: safeRCP gives FLT_MAX, values become 0.
    np.testing.assert_array_equal(cpu.normalize(np.array([1.0, 1.0])), [0.0, 0.0])


def test_alias_tables_reproduce_the_distribution():
    p = np.array([0.1, 0.2, 0.3, 0.4], np.float32)
    rc, alias, prob = cpu.build_alias(np.cumsum(p))
    assert rc == 0
    # Probability mass of each outcome under the alias method.
    n = len(p)
    mass = np.zeros(n)
    for k in range(n):
        mass[k] += prob[k] / n
        mass[alias[k]] += (1 - prob[k]) / n
    np.testing.assert_allclose(mass, p, atol=1e-6)
    assert cpu.build_alias(np.array([0.5, 0.4], np.float32))[0] == 1  # negative probability
    assert cpu.build_alias(np.array([0.5, 0.9], np.float32))[0] == 2  # does not sum to 1


def test_mis_scatter_walk_counts_the_steps_of_each_sample():
    """The scattering MIS oracle (transient_reconstruction.cuh:235-250) with a
    constant capture and every scan point at one place (so the drawn point
    does not change the path): per voxel it equals the single-bin MIS term
    times the number of steps of the walk, counted by a scalar loop."""
    from oracle import numpy_ref

    rng = np.random.default_rng(12)
    L, T = 16, 96
    lxyz = np.tile(np.array([[0.05, 0.0, -0.1]], np.float32), (L, 1))
    o = _info(L, T, 0.03, (3, 2, 4), (-0.4, -1.0, -0.4), (0.25, 0.05, 0.2))
    cube = np.full((L, T), 2.0, np.float32)
    cdf = np.cumsum(rng.uniform(0.5, 1.5, L)).astype(np.float32)
    cdf /= cdf[-1]
    rc, alias, prob = cpu.build_alias(cdf)
    assert rc == 0
    noise = rng.random(4096).astype(np.float32)
    one = numpy_ref.mis_reference(o, cube, lxyz, cdf, alias, prob, noise, 3)
    walk = numpy_ref.mis_reference(o, cube, lxyz, cdf, alias, prob, noise, 3, scatter=True)
    ext = 0.5 * np.sqrt(sum(float(v) ** 2 for v in o.voxel_size))
    step = float(o.time_step) + float(np.float32(1e-5))
    Vx, Vy, Vz = o.voxel_res
    counts = []
    for v in range(Vx * Vy * Vz):
        vz, rem = divmod(v, Vx * Vy)
        vy, vx = divmod(rem, Vx)
        p = np.array([o.hidden_min[0] + (vx + 0.5) * o.voxel_size[0], o.hidden_min[1] + (vz + 0.5) * o.voxel_size[1],
                      o.hidden_min[2] + (vy + 0.5) * o.voxel_size[2]])
        dist = 2.0 * np.linalg.norm(p - lxyz[0].astype(np.float64))
        d, k = max(0.0, dist - ext), 0
        while d < dist + ext and d / float(o.time_step) < T:
            k, d = k + 1, d + step
        assert walk.ravel()[v] == pytest.approx(k * one.ravel()[v], rel=1e-12)
        counts.append(k)
    assert min(counts) >= 2  # the walk visits several bins
    with pytest.raises(ValueError):
        numpy_ref.mis_reference(o, cube, lxyz, cdf, alias, prob, noise, 1, bins=np.zeros((24, L), np.int32),
                                scatter=True)


def test_mlp_oracle_gradient_matches_finite_differences():
    """The oracle's backward pass (exact FP64 mode) against central differences."""
    from oracle import mlp_ref

    rng = np.random.default_rng(0)
    p = np.zeros(mlp_ref.NPARAM)
    p[mlp_ref.OW1:mlp_ref.OB1] = (rng.uniform(-0.3, 0.3, (64, 32)) * (np.arange(32) < 19)).ravel()
    p[mlp_ref.OB1:] = rng.uniform(-0.2, 0.2, mlp_ref.NPARAM - mlp_ref.OB1)
    feats = rng.normal(size=(3, 10, mlp_ref.FEAT))
    q = rng.uniform(size=(3, 10))
    q /= q.sum(axis=1, keepdims=True)
    loss, grad = mlp_ref.loss_and_grad(p, feats, q, rounding=False)
    idx = np.concatenate([rng.choice(np.arange(mlp_ref.OW1, mlp_ref.OB1).reshape(64, 32)[:, :19].ravel(), 8),
                          rng.choice(np.arange(mlp_ref.OB1, mlp_ref.NPARAM), 24)])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mlp_ref.loss_and_grad(pp, feats, q, rounding=False)[0] -
              mlp_ref.loss_and_grad(pm, feats, q, rounding=False)[0]) / (2 * h)
        assert abs(fd - grad[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, grad[i])


def test_mlp_bf16_rounding_is_nearest_even():
    from oracle import mlp_ref

    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-3], np.float32)
    want = np.array([1.0, 1.0, 1.0078125, -2.5, 0.0030059814453125])
    np.testing.assert_array_equal(mlp_ref.bf16(x), want)


def test_splat_oracle_known_answer():
    """One scan point at the origin, one bin of path 1 m: a hemisphere of
    radius 0.5 below the wall; the pixel straight below the scan point lands
    at depth 0.5 m."""
    from types import SimpleNamespace

    info = SimpleNamespace(voxel_res=(5, 5, 10), voxel_size=(0.2, 0.1, 0.2), hidden_min=(-0.5, -1.0, -0.5),
                           time_step=0.25, time_offset=0.0)
    cube = np.zeros((1, 8), np.float32)
    cube[0, 4] = 3.0  # bin 4: path 1.0 m, radius 0.5 m
    vol = numpy_ref.splat_backproject(info, cube, np.zeros((1, 3), np.float32), grid=(5, 5))
    # Pixel (2, 2) is the centre (x = z = 0): y = -0.5 -> depth index (−0.5 + 1.0) / 0.1 = 5.
    assert vol[5, 2, 2] == pytest.approx(3.0)
    assert vol.sum() == pytest.approx(3.0 * np.count_nonzero(vol > 0) * 1.0)  # each fragment adds 3
    assert np.count_nonzero(vol) >= 5
