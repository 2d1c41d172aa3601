"""The reference's own golden vectors, replayed through libvkhel on the GPU.

Each operation recorded from the reference's test/vector.c
(tests/golden/reference_vectors.json) is run through the public C API with the
same call pattern: create vectors, copy_from_host, the operation, then read
the result back through map/unmap as test/vector.c:13-21 does.
"""
import numpy as np
import pytest

from conftest import load_golden, u64

pytestmark = pytest.mark.gpu

VEC = load_golden("reference_vectors.json")


def _ints(xs):
    return u64([int(x) for x in xs])


@pytest.mark.parametrize("i", range(len(VEC["ops"])), ids=lambda i: f"{i}-{VEC['ops'][i]['op']}")
def test_reference_vector(vk, ctx, i):
    op = VEC["ops"][i]
    p = {k: int(v) for k, v in op["params"].items()}
    name = op["op"]
    expect = _ints(op["expected"])
    a = vk.Vector(ctx, len(op["a"]))
    a.copy_from_host(_ints(op["a"]))
    if name == "copy_from_host":
        out = a
    elif name == "dup":
        out = a.dup()
    elif name in ("forward_transform", "inverse_transform"):
        t = vk.NttTables(p["n"], p["q"], p["w"])
        out = vk.Vector(ctx, p["n"])
        getattr(vk, name)(a, out, t)
    else:
        out = vk.Vector(ctx, len(expect))
        if name == "elemfma":
            b = vk.Vector(ctx, _ints(op["b"]))
            vk.elemfma(a, b, out, p["multiplier"], p["mod"])
        elif name == "elemmul":
            b = vk.Vector(ctx, _ints(op["b"]))
            vk.elemmul(a, b, out, p["mod"])
        elif name == "elemmod":
            vk.elemmod(a, out, p["mod"], p["q"])
        elif name == "elemgtadd":
            vk.elemgtadd(a, out, p["bound"], p["diff"])
        elif name == "elemgtsub":
            vk.elemgtsub(a, out, p["bound"], p["diff"], p["mod"])
    np.testing.assert_array_equal(out.map_read(), expect)


def test_reference_transform_in_place(vk, ctx):
    # test/vector.c:300-303 and 323-326: forward/inverse with operand == result
    ops = [o for o in VEC["ops"] if o["op"] in ("forward_transform", "inverse_transform")
           and o["params"]["n"] == "16"]
    assert len(ops) == 2
    for op in ops:
        p = {k: int(v) for k, v in op["params"].items()}
        t = vk.NttTables(p["n"], p["q"], p["w"])
        v = vk.Vector(ctx, _ints(op["a"]))
        getattr(vk, op["op"])(v, v, t)
        np.testing.assert_array_equal(v.map_read(), _ints(op["expected"]))


@pytest.mark.gpu
def test_vector_dbgprint_matches_reference_format(vk, ctx, capfd):
    # src/vector.c:237-247: the words, ", "-separated, then a newline
    import ctypes
    v = vk.Vector(ctx, np.array([3, 0, (1 << 64) - 1, 42], dtype=np.uint64))
    vk.lib().vkhel_vector_dbgprint(v.ptr)
    ctypes.CDLL(None).fflush(None)
    assert capfd.readouterr().out == f"3, 0, {(1 << 64) - 1}, 42\n"
