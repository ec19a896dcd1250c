"""Transform descriptor algebra and plan analysis, on the CPU.

The descriptor values are the doctests and assertions of the reference
(src/Transforms/Transforms.jl:100-106,121-137,162-193,222-233,247-259,273-283,
test/transforms.jl:19-143, src/global_params.jl:26-41); the plan analysis runs
through the C ABI's host-only pfgb_plan_query and is compared with the oracle.
"""
import numpy as np
import pytest

import pencilffts_gb300 as P
from helpers import to_oracle
from oracle import pencilfft_oracle as O

T = P.Transforms


def test_binv_doctests():
    assert repr(T.binv(T.FFT(), 42)) == "BFFT"
    assert repr(T.binv(T.BRFFT(9), 42)) == "RFFT"
    assert T.binv(T.RFFT(), 10) == T.BRFFT(10)
    assert T.binv(T.RFFT(), 11) == T.BRFFT(11)
    assert T.binv(T.FFT_(), 4) == T.BFFT_()
    assert T.binv(T.BFFT_(), 4) == T.FFT_()
    assert T.binv(T.NoTransform(), 42) == T.NoTransform()
    assert T.binv(T.R2R(T.REDFT01), 42) == T.R2R(T.REDFT10)
    assert T.binv(T.R2R_(T.REDFT01), 42) == T.R2R_(T.REDFT10)


def test_is_inplace_doctests():
    assert T.is_inplace(T.RFFT()) is False
    assert T.is_inplace(T.NoTransform_()) is True
    assert T.is_inplace(T.FFT_(), T.R2R_(T.REDFT01)) is True
    assert T.is_inplace(T.FFT(), T.R2R(T.REDFT01)) is False
    assert T.is_inplace(T.FFT(), T.R2R_(T.REDFT01)) is None
    F, F_ = T.FFT(), T.FFT_()
    assert T.is_inplace(F, F, F_) is None
    assert T.is_inplace(F, F_, F) is None
    assert T.is_inplace(F_, F, F_) is None
    assert T.is_inplace(F_, F_, F_) is True
    assert T.is_inplace(F, F, F) is False


def test_scale_factor_doctests():
    C = np.zeros((3, 4, 5), dtype=np.complex64)
    R = np.zeros((3, 4, 5), dtype=np.float64)
    assert T.scale_factor(T.FFT(), C) == 60
    assert T.scale_factor(T.BFFT(), C) == 60
    assert T.scale_factor(T.BFFT(), C, range(2, 4)) == 20
    assert T.scale_factor(T.RFFT(), R, 2) == 4
    assert T.scale_factor(T.RFFT(), R, range(2, 4)) == 20
    assert T.scale_factor(T.BRFFT(8), C) == 96
    assert T.scale_factor(T.BRFFT(9), C) == 108
    with pytest.raises(TypeError):
        T.scale_factor(T.RFFT(), C, range(2, 4))
    assert T.scale_factor(T.FFT(), np.zeros((3, 4), dtype=np.complex64)) == 12


def test_eltypes_doctests():
    assert T.eltype_input(T.FFT(), np.float32) == np.complex64
    assert T.eltype_input(T.RFFT(), np.float64) == np.float64
    assert T.eltype_input(T.R2R(T.REDFT01), np.float64) is None
    assert T.eltype_input(T.NoTransform(), np.float64) is None
    assert T.eltype_output(T.NoTransform(), np.float32) == np.float32
    assert T.eltype_output(T.RFFT(), np.float64) == np.complex128
    assert T.eltype_output(T.BRFFT(4), np.complex64) == np.float32
    with pytest.raises(P.ArgumentError, match="invalid input data type for FFT"):
        T.eltype_output(T.FFT(), np.float64)


def test_expand_dims_doctests():
    assert repr(T.expand_dims(T.RFFT(), 3)) == "(RFFT, FFT, FFT)"
    assert repr(T.expand_dims(T.BRFFT(4), 3)) == "(BFFT, BFFT, BRFFT{even})"
    assert repr(T.expand_dims(T.NoTransform(), 2)) == "(NoTransform, NoTransform)"
    assert repr(T.expand_dims(T.RFFT_(), 2)) == "(RFFT!, FFT!)"


def test_r2r_kinds():
    for k in (T.R2HC, T.HC2R):
        with pytest.raises(P.ArgumentError, match="unsupported r2r transform kind"):
            T.R2R(k)
        with pytest.raises(P.ArgumentError):
            T.R2R_(k)
    assert repr(T.R2R(T.REDFT00)) == "R2R{REDFT00}"
    assert T.kind(T.R2R(T.RODFT11)) == T.RODFT11


def test_length_output():
    size_in = (16, 12, 6)
    trs = (T.RFFT(), T.FFT(), T.FFT())
    out = tuple(T.length_output(t, n) for t, n in zip(trs, size_in))
    assert out == (9, 12, 6)
    binvs = tuple(T.binv(t, n) for t, n in zip(trs, size_in))
    assert binvs == (T.BRFFT(16), T.BFFT(), T.BFFT())
    assert tuple(T.length_output(t, n) for t, n in zip(binvs, out)) == size_in


# -- plan analysis through the C ABI (host only) ---------------------------------
CASES = [
    ((16, 32, 64), T.RFFT(), np.float64, True, ()),
    ((64, 32, 128), (T.RFFT(), T.FFT(), T.FFT()), np.float64, True, ()),
    ((16, 12, 6), T.FFT(), np.float32, True, (3,)),
    ((16, 12, 6), T.BRFFT((16, 12, 6)), np.float64, True, ()),
    ((12, 13, 9), T.BRFFT((12, 13, 17)), np.float64, True, ()),
    ((16, 12, 6), (T.NoTransform(), T.RFFT(), T.FFT()), np.float64, True, ()),
    ((9, 7, 5, 12), T.RFFT(), np.float64, False, ()),
    ((11, 15), T.FFT_(), np.float64, True, ()),
    ((42, 24, 16), T.RFFT_(), np.float64, True, ()),
    ((512, 512, 257), (T.RFFT(), T.FFT(), T.R2R(T.REDFT00)), np.float64, True, ()),
    ((16, 12, 6), T.NoTransform(), np.float32, True, ()),
    ((16, 12, 6), T.NoTransform_(), np.float32, True, ()),
] + [((16, 12, 6), T.R2R(k), np.float64, True, ()) for k in T.R2R_SUPPORTED_KINDS]


@pytest.mark.parametrize("dims,tr,real,permute,edims", CASES)
def test_plan_query_matches_oracle(dims, tr, real, permute, edims):
    info = P.plan_query(dims, tr, real, permute_dims=permute, extra_dims=edims)
    trs = T.expand_dims(tr, len(dims)) if isinstance(tr, T.AbstractTransform) else tr
    orc = O.OraclePlan(dims, tuple(to_oracle(t) for t in trs), real, permute, edims)
    N = len(dims)
    assert tuple(info.dims_out[n] for n in range(N)) == orc.dims_out
    assert info.scale_factor == orc.scale
    assert bool(info.eltype_in_complex) == (orc.eltype_in.kind == "c")
    assert bool(info.eltype_out_complex) == (orc.eltype_out.kind == "c")
    perm = tuple(info.perm_out[q] for q in range(N))
    assert perm == (tuple(range(N - 1, -1, -1)) if (permute and N > 1) else tuple(range(N)))
    rb = np.dtype(real).itemsize
    ext = int(np.prod(edims)) if edims else 1
    nin = int(np.prod(dims)) * ext * (2 * rb if info.eltype_in_complex else rb)
    nout = int(np.prod(orc.dims_out)) * ext * (2 * rb if info.eltype_out_complex else rb)
    if info.inplace and isinstance(trs[0], T.RFFT):
        nin = 2 * (dims[0] // 2 + 1) * int(np.prod(dims[1:])) * ext * rb
    assert info.input_bytes == nin
    assert info.output_bytes == nout
    assert info.inplace == int(T.is_inplace(*trs))


def test_scale_factor_examples():
    # Parseval normalisation of test/rfft.jl:37: scale == Ngrid
    assert P.plan_query((42, 24, 16), T.RFFT()).scale_factor == 42 * 24 * 16
    assert P.plan_query((41, 23, 15), T.RFFT()).scale_factor == 41 * 23 * 15
    # REDFT00 along z of length 257 has logical size 2*(257-1) = 512
    info = P.plan_query((512, 512, 257), (T.RFFT(), T.FFT(), T.R2R(T.REDFT00)))
    assert info.scale_factor == 512 * 512 * 512


@pytest.mark.parametrize("bad,match", [
    (dict(dims=(10, 8), tr=(T.FFT(), T.FFT_())), "cannot combine in-place and out-of-place"),
    (dict(dims=(10, 8), tr=(T.FFT(), T.RFFT())), "invalid input data type"),
    (dict(dims=(10, 8), tr=(T.RFFT(), T.RFFT())), "invalid input data type"),
    (dict(dims=(1, 8), tr=(T.R2R(T.REDFT00), T.FFT())), "REDFT00"),
    (dict(dims=(0, 8), tr=T.FFT()), "positive"),
])
def test_plan_query_errors(bad, match):
    with pytest.raises(P.ArgumentError, match=match):
        P.plan_query(bad["dims"], bad["tr"])


def test_global_params_doctest():
    """reference src/global_params.jl:26-41."""
    info = P.plan_query((64, 32, 128), (T.RFFT(), T.FFT(), T.FFT()))
    assert tuple(info.dims_out[n] for n in range(3)) == (33, 32, 128)
    assert not info.eltype_in_complex


def test_input_data_type():
    """reference test/transforms.jl:362-379."""
    assert P.plan_query((8, 6), (T.NoTransform(), T.FFT()), np.float32).eltype_in_complex
    assert not P.plan_query((8, 6), (T.NoTransform(), T.NoTransform()), np.float32).eltype_in_complex


def test_tc_split_precision_descriptor():
    """The tensor-core split form is a Float32-only precision mode."""
    P.plan_query((64, 512, 256), T.FFT(), np.float32, precision="tc")
    with pytest.raises(P.ArgumentError, match="Float32"):
        P.plan_query((64, 512, 256), T.FFT(), np.float64, precision="tc")
    with pytest.raises(P.ArgumentError, match="precision"):
        P.plan_query((8, 8), T.FFT(), np.float32, precision="bf16")


def test_block_float_precision_descriptor():
    """The block floating point form is a Float64-only precision mode."""
    P.plan_query((64, 512, 256), T.RFFT(), np.float64, precision="fx")
    with pytest.raises(P.ArgumentError, match="Float64"):
        P.plan_query((64, 512, 256), T.FFT(), np.float32, precision="fx")


def test_fftw_flags_select_measurement():
    """FFTW.ESTIMATE (the reference's default) plans without measuring; any
    other planner flag, or autotune=True, measures."""
    from pencilffts_gb300.plans import _autotune_from
    assert _autotune_from(None, None) == 0
    assert _autotune_from(P.FFTW_ESTIMATE, None) == 0
    assert _autotune_from(P.FFTW_MEASURE, None) == 1
    assert _autotune_from(P.FFTW_PATIENT, None) == 1
    assert _autotune_from(P.FFTW_ESTIMATE, True) == 1
    assert _autotune_from(P.FFTW_MEASURE, False) == 0
    P.plan_query((64, 48, 32), T.RFFT())  # host-only analysis never measures


def test_long_c2c_lines_take_two_passes():
    """c2c lines above 4096 points are split in two register passes (host
    plan query, no device)."""
    info = P.plan_query((16384,), T.FFT(), np.float64)
    assert info.n_passes_forward == 2 and info.n_passes_backward == 2
    info = P.plan_query((8, 1 << 20), T.FFT(), np.float32)
    assert info.n_passes_forward == 3


def test_long_lines_pass_counts():
    """Host plan query of lines beyond one pass: r2c / c2r lines above 4096
    points as a pack map, the two passes of the packed c2c line and a
    separating map; c2c lines without a split as a Bluestein convolution
    (chirp map, two split transforms, filter product, chirp map; r2c lines
    add their pack and separating maps); R2R lines as a gathering map, the
    extension's c2c passes and an output map.  Beyond 2^23 points without a
    split a line stays unsupported."""
    for dims, tr, np_ in (((16384,), T.RFFT(), 4), ((8193,), T.BRFFT(16384), 4),
                          ((5000, 6), T.RFFT(), 5), ((1 << 20,), T.RFFT(), 4),
                          ((8209,), T.FFT(), 7), ((8209,), T.RFFT(), 9),
                          ((5000,), T.R2R(T.REDFT10), 4), ((4099,), T.R2R(T.REDFT11), 9)):
        info = P.plan_query(dims, tr, np.float64)
        assert info.n_passes_forward == np_ and info.n_passes_backward == np_, dims
    with pytest.raises(P.LibraryError):
        P.plan_query(((1 << 23) + 9,), T.FFT(), np.float64)
    # more than 12 passes: the scratch buffers alternate (no exhaustive search)
    info = P.plan_query((4097, 4099), T.FFT(), np.float32)
    assert info.n_passes_forward == 14 and info.scratch_bytes > 0
