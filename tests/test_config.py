"""Configuration and host-side failure handling through the C ABI.

Every case here fails (or passes configuration) before the engine's first CUDA
call, so it runs without a GPU: a missing or garbled key, an unsupported wall
axis, a truncated / oversized / NaN-carrying dump.  The reference would throw
an uncaught std::invalid_argument or exit(2) instead (src/config.h:45-50,
src/dugks.cu:360-374)."""
import os

import numpy as np
import pytest

import pydugks
from pydugks import DG_ERR_CONFIG, DG_ERR_CUDA, DG_ERR_IO, DG_ERR_NUMERIC, DG_ERR_UNSUPPORTED, DugksError


def create(text, workdir="."):
    try:
        e = pydugks.Engine(text, workdir=workdir)
    except DugksError as err:
        return err.code, str(err)
    e.close()
    return 0, ""


def gpu_or_ok(code):
    # a valid configuration either builds an engine (GPU present) or stops at the first CUDA call
    return code in (0, DG_ERR_CUDA)


def test_valid_reference_config_parses():
    code, msg = create(pydugks.make_config())
    assert gpu_or_ok(code), msg


@pytest.mark.parametrize("key", pydugks.REFERENCE_KEYS)
def test_missing_key_is_config_error(key):
    text = "\n".join(l for l in pydugks.make_config().splitlines() if not l.startswith(key + "="))
    code, msg = create(text)
    assert code == DG_ERR_CONFIG, (key, code, msg)
    assert key in msg


def test_garbled_value_is_config_error():
    code, msg = create(pydugks.make_config(nx="abc"))
    assert code == DG_ERR_CONFIG and "nx" in msg
    code, msg = create(pydugks.make_config(visc="x0.1"))
    assert code == DG_ERR_CONFIG


def test_stoi_stof_semantics():
    # leading blanks and trailing junk are accepted like std::stoi / std::stof
    code, msg = create(pydugks.make_config(nx=" 64 # wall-normal", CFL="0.7abc"))
    assert gpu_or_ok(code), msg


def test_first_occurrence_wins_and_comments_ignored():
    text = pydugks.make_config() + "nx=abc\n# a comment line without the separator\n"
    code, msg = create(text)
    assert gpu_or_ok(code), msg


def test_key_with_trailing_blank_is_not_the_key():
    text = pydugks.make_config().replace("\nnx=64", "\nnx =64")
    code, msg = create(text)
    assert code == DG_ERR_CONFIG and "nx" in msg


def test_unsupported_wall_axis():
    code, msg = create(pydugks.make_config(periods_y=0))
    assert code == DG_ERR_UNSUPPORTED
    code, msg = create(pydugks.make_config(periods_z=0))
    assert code == DG_ERR_UNSUPPORTED


def test_unknown_case_without_restart():
    code, msg = create(pydugks.make_config(case="nonsense"))
    assert code == DG_ERR_CONFIG and "Unknown case" in msg


def test_bad_extension_values():
    assert create(pydugks.make_config(precision="fp8"))[0] == DG_ERR_CONFIG
    assert create(pydugks.make_config(mesh="cubic"))[0] == DG_ERR_CONFIG
    assert create(pydugks.make_config(mesh="tanh", mesh_alpha=1.5))[0] == DG_ERR_CONFIG
    assert create(pydugks.make_config(mesh="tanh", periods_x=1))[0] == DG_ERR_CONFIG
    assert create(pydugks.make_config(precision="bf16", rounding="up"))[0] == DG_ERR_CONFIG
    assert gpu_or_ok(create(pydugks.make_config(precision="bf16", rounding="nearest"))[0])
    assert create(pydugks.make_config(precision="fp16", rounding="down"))[0] == DG_ERR_CONFIG
    assert gpu_or_ok(create(pydugks.make_config(precision="fp16", rounding="stochastic"))[0])


def test_tiny_grid_rejected():
    assert create(pydugks.make_config(nx=2))[0] < 0


def _write_dump(tmp_path, step, arr):
    arr.tofile(os.path.join(tmp_path, "ddf%08d.dat" % step))


def test_restart_missing_dump(tmp_path):
    code, msg = create(pydugks.make_config(restart=1, nrestart=7, nx=8, ny=4, nz=2), workdir=str(tmp_path))
    assert code == DG_ERR_IO and "ddf00000007.dat" in msg


def test_restart_truncated_dump(tmp_path):
    _write_dump(tmp_path, 3, np.zeros(19 * 8 * 4 * 2 - 1))
    code, msg = create(pydugks.make_config(restart=1, nrestart=3, nx=8, ny=4, nz=2), workdir=str(tmp_path))
    assert code == DG_ERR_IO and "bytes" in msg


def test_restart_oversized_dump(tmp_path):
    _write_dump(tmp_path, 3, np.zeros(19 * 8 * 4 * 2 + 19))
    code, msg = create(pydugks.make_config(restart=1, nrestart=3, nx=8, ny=4, nz=2), workdir=str(tmp_path))
    assert code == DG_ERR_IO


def test_restart_nan_dump(tmp_path):
    a = np.full(19 * 8 * 4 * 2, 1.0 / 19)
    a[100] = np.nan
    _write_dump(tmp_path, 3, a)
    code, msg = create(pydugks.make_config(restart=1, nrestart=3, nx=8, ny=4, nz=2), workdir=str(tmp_path))
    assert code == DG_ERR_NUMERIC


def test_restart_fp32_dump_width(tmp_path):
    # a PREC4-width dump (4-byte reals) is accepted by an fp32 engine and rejected by an fp64 one
    a = np.full(19 * 8 * 4 * 2, 1.0 / 19, dtype=np.float32)
    _write_dump(tmp_path, 5, a)
    code, _ = create(pydugks.make_config(restart=1, nrestart=5, nx=8, ny=4, nz=2, precision="fp32"),
                     workdir=str(tmp_path))
    assert gpu_or_ok(code)
    code, _ = create(pydugks.make_config(restart=1, nrestart=5, nx=8, ny=4, nz=2), workdir=str(tmp_path))
    assert code == DG_ERR_IO


def test_null_arguments():
    L = pydugks.lib()
    assert L.dg_step(None, 1) == pydugks.DG_ERR_ARG
    assert L.dg_destroy(None) == pydugks.DG_ERR_ARG
    assert L.dg_create_from_text(None, None, None) == pydugks.DG_ERR_ARG
