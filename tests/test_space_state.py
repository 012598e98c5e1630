"""The EXRBTQ31 space state (RaBitQSpace::saveState / loadState, space_rabitq.h:3139-3345) against
states the reference itself saved (tests/golden/space_states.npz): same bytes written, same
fields read, and bytes written here accepted by the reference's own loader."""
import numpy as np
import pytest

from conftest import load_golden

NAMES = ["kernels_d128", "kernels_d960", "kernels_d1536"]


@pytest.mark.parametrize("name", NAMES)
def test_writer_matches_reference_bytes(oracle, name):
    from quantization_graph_gb300 import space_state

    g = load_golden(name)
    ref = load_golden("space_states")[name].tobytes()
    dim = int(g["dim"])
    o = oracle.Oracle(dim, g["center"])
    buf = space_state.state_bytes(dim, 100, g["center"], o.signs())
    assert buf == ref
    st = space_state.parse_state(ref)
    assert st["dim"] == dim and st["seed"] == 100 and st["code_dim"] == o.D
    np.testing.assert_array_equal(st["center"], np.asarray(g["center"], np.float32))
    np.testing.assert_array_equal(st["signs"], o.signs())
    if oracle.reference_available():  # the reference's loader takes what this writer wrote
        r = oracle.Reference(dim, np.zeros(dim, np.float32))
        assert r.load_state(buf)
        assert r.save_state() == ref


def test_reader_refuses_other_layouts():
    from quantization_graph_gb300 import space_state

    ref = load_golden("space_states")["kernels_d128"].tobytes()
    with pytest.raises(ValueError):
        space_state.parse_state(b"EXRBTQ22" + ref[8:])
    bad = bytearray(ref)
    bad[8 + 8 + 8 + 4 + 4 + 4 + 8 + 8 + 8 + 8] = 3  # residual bits 3
    with pytest.raises(ValueError):
        space_state.parse_state(bytes(bad))
    with pytest.raises(ValueError):
        space_state.parse_state(ref[:200])


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_library_save_and_load(cuda, name):
    """A space of the library saves the reference's bytes; the reference's state loads into the
    library and encodes the fixture's vectors to the reference's records."""
    from cases import kernel_inputs
    from quantization_graph_gb300 import space_state
    from quantization_graph_gb300.space import RabitqSpace

    g = load_golden(name)
    ref = load_golden("space_states")[name].tobytes()
    sp = RabitqSpace(int(g["dim"]), g["center"])
    assert space_state.save_state(sp) == ref
    loaded = space_state.load_state(ref)
    X, _ = kernel_inputs(int(g["dim"]), int(g["n"]), int(g["nq"]), int(g["seed"]))
    compact, residual = loaded.encode(cuda.from_numpy(X).cuda())
    np.testing.assert_array_equal(compact.cpu().numpy(), g["compact"])
    np.testing.assert_array_equal(residual.cpu().numpy(), g["residual"])
    assert space_state.save_state(loaded) == ref
