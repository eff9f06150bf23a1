"""CPU-side checks of the C ABI: the libraries build, load, and export every
entry point include/phx_fluid.h and include/phx_radiation.h declare; the
ctypes mirror matches the headers.  No compute calls (no GPU here)."""
import re
import subprocess
from pathlib import Path

import pytest

from phoebus_gb300 import abi

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "phx_fluid.h"
HEADERS = [HEADER, ROOT / "include" / "phx_radiation.h"]


def declared_functions():
    text = "".join(h.read_text() for h in HEADERS)
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(phx_[a-z0-9_]+)\s*\(", text)))


def test_header_and_ctypes_agree():
    assert declared_functions() == abi.exported_symbols()


@pytest.mark.parametrize("exact", [False, True])
def test_library_exports_every_symbol(built, exact):
    path = abi.lib_path(exact)
    assert path.exists()
    out = subprocess.run(["nm", "-D", "--defined-only", str(path)], capture_output=True, text=True, check=True).stdout
    syms = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [f for f in declared_functions() if f not in syms]
    assert not missing, f"not exported: {missing}"


def test_library_loads_without_gpu(built):
    # dlopen + symbol binding works without a device; only pure host calls.
    lib = abi.load(False)
    assert lib.phx_abi_version() == 1
    assert lib.phx_build_exact() == 0
    assert abi.load(True).phx_build_exact() == 1
    p = abi.Params()
    lib.phx_params_default(p)
    ref = abi.default_params()
    for name, _ in abi.Params._fields_:
        assert getattr(p, name) == getattr(ref, name), name
    g = abi.Geometry()
    lib.phx_geometry_default(g, abi.GEOM_FMKS)
    gr = abi.default_geometry(abi.GEOM_FMKS)
    for name in ("hslope", "poly_xt", "poly_alpha", "smooth", "hexp_br", "derefine_poles"):
        assert getattr(g, name) == getattr(gr, name), name
    assert lib.phx_status_string(2) == b"con2prim root not bracketed"
    o = abi.MlpTrainOpts()
    lib.phx_mlp_train_opts_default(o)
    ref_o = abi.default_train_opts()
    for name, _ in abi.MlpTrainOpts._fields_:
        assert getattr(o, name) == getattr(ref_o, name), name


def test_struct_sizes_match_header(built, tmp_path):
    """Compile a tiny C program against the header and compare sizeof/offsets
    with the ctypes mirror."""
    import ctypes as C

    src = tmp_path / "sz.c"
    fields = {"phx_params": abi.Params, "phx_block": abi.BlockS, "phx_geometry": abi.Geometry,
              "phx_c2p_stats": abi.C2PStats, "phx_mlp_train_opts": abi.MlpTrainOpts, "phx_mesh": abi.Mesh,
              "phx_rad_params": abi.RadParams, "phx_rad_block": abi.RadBlockS}
    lines = ['#include <stdio.h>', '#include <stddef.h>'] + [f'#include "{h}"' for h in HEADERS] + ["int main(void){"]
    for cname, cls in fields.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0;}")
    src.write_text("\n".join(lines))
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-o", str(exe), str(src)], check=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True).stdout.splitlines())
    for cname, cls in fields.items():
        assert int(out[cname]) == C.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert int(out[f"{cname}.{fname}"]) == getattr(cls, fname).offset, f"{cname}.{fname}"


def _has_cuda():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_cuda(), reason="checks the no-device path")
def test_context_without_device_fails_loudly(built):
    """No GPU: creating a context returns PHX_ERR_NO_DEVICE and the Python
    layer raises; there is no CPU fallback."""
    from phoebus_gb300.fluid import FluidContext

    with pytest.raises(abi.PhxError) as e:
        FluidContext(0)
    assert e.value.status == 6 and "no CUDA device" in str(e.value)


def test_status_strings(built):
    lib = abi.load(False)
    for code, text in abi.STATUS.items():
        got = lib.phx_status_string(code).decode()
        assert got == text, (code, got)
