"""The allocation-free game_of_life entry point, sg_gol_steps_noalloc.

Callers that cannot call cudaMalloc (a host program whose device memory belongs
to another allocator, or a loop that must not allocate between steps) advance a
board held in their own device buffers; the library's only working memory is a
static device array of fixed size.  This checks the entry point through the
C-ABI against the regular entry points (build_state + run), bit for bit (the
same bar as every game_of_life test), on two calls in a row.  The file sorts
last so that a run stopping at the first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_CELLS = 1 << 20


def gol_net(rows, cols):
    return {"structures": [{"name": "g", "type": "parallel", "layers": [
        {"name": "board", "neural model": "game_of_life", "rows": rows, "columns": cols,
         "survival_min": 2, "survival_max": 3, "birth_min": 3, "birth_max": 3}]}],
        "connections": [{"name": "nbr", "from layer": "board", "to layer": "board",
                         "type": "convergent", "convolutional": True, "plastic": False,
                         "opcode": "add",
                         "weight config": {"type": "flat", "weight": 1.0, "diagonal": False},
                         "arborized config": {"field size": 3, "wrap": True}}]}


@pytest.fixture(scope="module")
def lib():
    from synaptogenesis_gb300 import syngen
    assert syngen.get_gpus(), "no CUDA GPU visible"
    L = ctypes.CDLL(syngen.LIB_PATH)
    L.sg_gol_steps_noalloc.restype = ctypes.c_int
    L.sg_gol_steps_noalloc.argtypes = (
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
        ctypes.c_void_p)
    return L


def test_noalloc_matches_regular_entry_points_on_two_calls(lib):
    import torch
    from synaptogenesis_gb300 import syngen
    syngen.set_warnings(False)
    rows, cols = 300, 500
    board = np.random.default_rng(9).integers(0, 2**32, rows * cols, dtype=np.uint64).astype(np.uint32)
    kernel = np.array([1, 1, 1, 1, 0, 1, 1, 1, 1], np.float32)

    d_words = torch.from_numpy(board.view(np.int32).copy()).cuda()
    d_input = torch.zeros(rows * cols, dtype=torch.float32, device="cuda")
    d_w = torch.from_numpy(kernel).cuda()
    stream = torch.cuda.current_stream()

    net = syngen.Network(gol_net(rows, cols))
    net.build_state()
    net.get_neuron_data("g", "board", "output").to_np_array().view(np.uint32)[:] = board
    env = syngen.Environment({"modules": []})

    for steps in (13, 10):
        rc = lib.sg_gol_steps_noalloc(d_words.data_ptr(), d_input.data_ptr(), rows, cols,
                                      d_w.data_ptr(), 3, steps, 2, 3, 3, 3,
                                      ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0
        torch.cuda.synchronize()
        report = net.run(env, {"iterations": steps})
        assert report.obj is not None, syngen.last_error()
        want_words = net.get_neuron_data("g", "board", "output").to_np_array().view(np.uint32)
        want_input = net.get_neuron_data("g", "board", "input").to_np_array()
        got_words = d_words.cpu().numpy().view(np.uint32)
        got_input = d_input.cpu().numpy()
        assert np.array_equal(got_words, want_words)
        assert np.array_equal(got_input, want_input)


def test_noalloc_rejects_boards_beyond_its_scratch(lib):
    import torch
    d = torch.zeros(16, dtype=torch.int32, device="cuda")
    w = torch.ones(9, dtype=torch.float32, device="cuda")
    rc = lib.sg_gol_steps_noalloc(d.data_ptr(), None, 1024, 1025, w.data_ptr(), 3, 1,
                                  2, 3, 3, 3, None)
    assert rc == -2 and 1024 * 1025 > MAX_CELLS
    rc = lib.sg_gol_steps_noalloc(d.data_ptr(), None, 4, 4, w.data_ptr(), 5, 1, 2, 3, 3, 3, None)
    assert rc == -1
