"""The tensor-core contraction (BF16 hi/lo split, tcgen05) through the C-ABI,
against the FP64 oracle and the FP32 CUDA-core path.

Parity bar (floating point, as for the FP32 path): peak values within 1e-4
relative of the FP64 oracle; the same best (ref, angle, sx, sy, mirror) for
>= 99.5% of particles (angle compared circularly within ANGLE_TOL degrees);
all (ref, particle) tuples >= 99%.

Shapes cover the kernels' tiling: an odd ring-group count (a zero K group
in shared memory), 61 rings (4 K steps), shift grids of 1, 25, 49, 81 and
121 shifts (one to three shift blocks), more than 128 references (two
reference tiles, the last partial), fractional base shifts, one particle.
"""
import numpy as np
import pytest

from gpuisac import synth

from test_gpu_align import ANGLE_TOL, PEAK_RTOL, circ_diff, compare, oracle_run

pytestmark = pytest.mark.gpu


def split_align(st, NR, rng, base=None):
    from gpuisac import multi_ref_align
    P, R = st.particles.shape[0], st.refs.shape[0]
    pl, d = multi_ref_align(st.particles, st.refs, NR, rng, rng, base_shifts=base, contraction_mode="bf16x3")
    return pl.reshape(R, P, 4), d


@pytest.mark.parametrize("P,R,D,NR,rng", [
    (40, 12, 64, 29, 2.0),    # the 64^2 / 29-ring shape: 25 shifts, 4 K groups
    (24, 9, 76, 35, 3.0),     # the 76^2 / 35-ring shape: 49 shifts, 5 K groups (zero group)
    (6, 5, 128, 61, 4.0),     # the 128^2 / 61-ring shape: 81 shifts in two blocks, 8 K groups
    (5, 3, 64, 20, 5.0),      # 121 shifts in three blocks
    (1, 1, 48, 1, 0.0),       # one ring, one shift, one particle, one reference
])
def test_split_matches_oracle(gpulib, cuda, oracle_mod, P, R, D, NR, rng):
    st = synth.make_stack(P, D, R, int(rng), 0.1, D * 0.4, 900 + P + NR)
    peak_g, d = split_align(st, NR, rng)
    peak_o, d_o = oracle_run(oracle_mod, st.particles, st.refs, NR, rng, tex=gpulib.get_texture_limit(D))
    compare(peak_g, d, peak_o, d_o)


def test_split_two_reference_tiles_and_base_shifts(gpulib, cuda, oracle_mod):
    """150 references: two tiles of 75 (N = 160 columns each), fractional base shifts."""
    st = synth.make_stack(12, 64, 150, 1, 0.1, 26.0, 910)
    base = np.random.default_rng(3).uniform(-1.4, 1.4, (12, 2)).astype(np.float32)
    peak_g, d = split_align(st, 29, 1.0, base=base)
    peak_o, d_o = oracle_run(oracle_mod, st.particles, st.refs, 29, 1.0, base=base,
                             tex=gpulib.get_texture_limit(64))
    compare(peak_g, d, peak_o, d_o)


def test_split_close_to_fp32_path(gpulib, cuda):
    """Device entry point, both contractions on the same resident stacks: peak
    values within 1e-4 relative, tuples (nearly) all the same."""
    import torch

    from gpuisac import multi_ref_align_device
    st = synth.make_stack(200, 76, 40, 3, 0.05, 34.0, 911)
    parts, refs = torch.from_numpy(st.particles).to(cuda), torch.from_numpy(st.refs).to(cuda)
    d32, p32 = multi_ref_align_device(parts, refs, 35, 3.0, 3.0, contraction_mode="fp32")
    d32, p32 = d32.cpu().numpy(), p32.cpu().numpy()
    d16, p16 = multi_ref_align_device(parts, refs, 35, 3.0, 3.0, contraction_mode="bf16x3")
    d16, p16 = d16.cpu().numpy(), p16.cpu().numpy()
    rel = np.abs(d16.astype(np.float64) - d32) / np.maximum(np.abs(d32), 1e-30)
    assert rel.max() <= PEAK_RTOL, rel.max()
    same = (p16[..., 1:] == p32[..., 1:]).all(-1) & (circ_diff(p16[..., 0], p32[..., 0]) < ANGLE_TOL)
    assert same.mean() >= 0.99, same.mean()
    assert (d16.argmax(0) == d32.argmax(0)).mean() >= 0.995


def test_contraction_mode_switch(gpulib, cuda):
    from gpuisac import contraction
    assert gpulib.gpuisac_get_contraction() == 0
    with contraction("bf16x3"):
        assert gpulib.gpuisac_get_contraction() == 1
    assert gpulib.gpuisac_get_contraction() == 0
    assert gpulib.gpuisac_set_contraction(7) == -1
    gpulib.gpuisac_clear_error()
