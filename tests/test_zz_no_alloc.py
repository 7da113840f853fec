"""The allocation-free QR entry point (rsvdt_qr_all_freqs_noalloc) against
the context's QRAllFreqs (rsvdt_qr_all_freqs), through the C ABI.

rsvdt_qr_all_freqs_noalloc is for callers that cannot call cudaMalloc
(a stream capture open elsewhere, a host framework that owns all device
memory through its own pool, a service that forbids allocation after
start-up): the caller passes device input and output, and the scratch comes
from a fixed device array inside the library. This file is collected last
so that a run stopping at the first failure has run every other test first.
"""
import numpy as np
import pytest

from rsvdt import synth

pytestmark = pytest.mark.gpu

TOL = 1e-11  # same CholQR passes, different row chunking of the Gram sums


def _reference_q(Y, nw, k):
    """QR through a context (the existing entry point)."""
    import rsvdt
    rows = Y.shape[0]
    ctx = rsvdt.Context(rsvdt.default_params(k=k, Nw=nw, w=0.1, dt=0.5, TransientLength=0.0, Display=0))
    ctx.set_operator(synth.gl_operator(rows, mu0=0.2))
    ctx.set_sketch(Y)
    ctx.qr_all_freqs()
    Q = ctx.get_block()
    ctx.close()
    return Q


def _noalloc_q(Y, nw, k, torch, in_place=False):
    """QR through rsvdt_qr_all_freqs_noalloc on torch-allocated device
    buffers (the caller allocates; the entry point does not), issued on a
    non-blocking stream of the caller's own."""
    import rsvdt
    rows = Y.shape[0]
    host = np.ascontiguousarray(Y).view(np.float64)  # [row][iw*k + j] (re, im)
    d_in = torch.from_numpy(host.copy()).cuda()
    d_out = d_in if in_place else torch.empty_like(d_in)
    torch.cuda.synchronize()
    stream = torch.cuda.Stream()
    rsvdt.qr_all_freqs_noalloc(d_in.data_ptr(), d_out.data_ptr(), rows, nw, k, stream.cuda_stream)
    out = d_out.cpu().numpy().view(np.complex128).reshape(rows, nw * k)
    return np.asfortranarray(out)


def test_noalloc_qr_matches_context_qr(built_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    # Calls in a row with different sizes and data: each call reuses the
    # scratch array the previous one left behind. The third case has more
    # Gram row chunks than the scratch holds (nw*k*k = 16384: at most 13
    # partial sets for 15 chunks of 2048 rows), so the rows are regrouped
    # into 13 longer chunks; it also runs in place (output = input).
    for rows, nw, k, seed, in_place in [(3000, 8, 4, 1, False), (5000, 16, 10, 2, False),
                                        (30000, 64, 16, 3, True)]:
        Y = synth.complex_normal(rows, nw * k, seed)
        Y[:, 0] *= 1e-3  # an ill-conditioned block
        Qref = _reference_q(Y, nw, k)
        Q = _noalloc_q(Y, nw, k, torch, in_place=in_place)
        err = np.linalg.norm(Q - Qref) / np.linalg.norm(Qref)
        assert err < TOL, (rows, nw, k, err)
        for iw in range(nw):
            b = Q[:, iw * k:(iw + 1) * k]
            assert np.abs(b.conj().T @ b - np.eye(k)).max() < 1e-12


def test_noalloc_reports_rank_deficient_block(built_lib):
    import rsvdt
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    rows, nw, k = 2000, 4, 6
    Y = synth.complex_normal(rows, nw * k, 5)
    Y[:, 2 * k + 3] = 0  # frequency 2 has a zero column
    with pytest.raises(rsvdt.RsvdtError) as e:
        _noalloc_q(Y, nw, k, torch)
    assert e.value.status == rsvdt.ERR_NOT_SPD
    # The flag of the failed call does not leak into the next one.
    Y[:, 2 * k + 3] = synth.complex_normal(rows, 1, 6)[:, 0]
    Q = _noalloc_q(Y, nw, k, torch)
    Qref = _reference_q(Y, nw, k)
    assert np.linalg.norm(Q - Qref) / np.linalg.norm(Qref) < TOL


def test_noalloc_rejects_oversized_blocks(built_lib):
    import rsvdt
    # nw*k*k = 64*32*32 = 65536 exceeds the fixed scratch (limit 65535);
    # rejected on the host before any device work, so null pointers are
    # never dereferenced.
    with pytest.raises(rsvdt.RsvdtError) as e:
        rsvdt.qr_all_freqs_noalloc(1, 1, 100, 64, 32, None)
    assert e.value.status == rsvdt.ERR_ARG
    assert "scratch" in str(e.value)
