"""Import the reference minkasi package in this container (fixture generation only).

The reference imports astropy, jax and matplotlib at module level; none is
installed here, so minimal stand-ins are registered in ``sys.modules`` before
the import.  None of the stubbed functionality is on the paths the fixtures
exercise (projections, NoiseSmoothedSVD, TodVec.dot, make_hits, run_pcg,
fft_r2r, truncate_tod): the WCS/FITS classes raise if called, and the scipy
DCT backend of ``minkasi/tools/py_fft.py`` is what the transform resolves to.
``libminkasi.so`` is the reference's own C, compiled from its source by
``make -C oracle ref REF_ROOT=<the reference checkout>``.

The reference checkout is named by the environment variable
MINKASI_REF_ROOT (the directory that holds ``minkasi/``); there is no
default, so running the fixture script states where the reference is:
``MINKASI_REF_ROOT=<checkout> python tests/golden/make_golden.py``.

This module is only used by ``make_golden.py``; nothing under tests/ that runs
on a GPU machine imports it.
"""
import ctypes
import os
import sys
import types

REF_ROOT = os.environ.get("MINKASI_REF_ROOT")
if not REF_ROOT:
    raise RuntimeError("set MINKASI_REF_ROOT to the reference checkout (the directory holding minkasi/)")
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def _stub(name, **attrs):
    m = types.ModuleType(name)
    m.__dict__.update(attrs)
    sys.modules[name] = m
    return m


class _Unavailable:
    def __init__(self, *a, **k):
        raise RuntimeError("astropy is not installed; this stub must not be called")


def install_stubs():
    astropy = _stub("astropy")
    wcs = _stub("astropy.wcs", WCS=_Unavailable)
    io = _stub("astropy.io")
    fits = _stub("astropy.io.fits", Header=_Unavailable, PrimaryHDU=_Unavailable,
                 open=_Unavailable, getdata=_Unavailable, getheader=_Unavailable)
    astropy.wcs, astropy.io, io.fits = wcs, io, fits
    import numpy as np
    jax = _stub("jax")
    jax.config = types.SimpleNamespace(update=lambda *a, **k: None)
    jnp = _stub("jax.numpy", fft=np.fft)
    jax.numpy = jnp
    mpl = _stub("matplotlib")
    plt = _stub("matplotlib.pyplot")
    mpl.pyplot = plt


def import_reference():
    """Return the imported ``minkasi`` package of the reference tree."""
    lib = os.path.join(REPO, "oracle", "_ref", "libminkasi.so")
    if not os.path.exists(lib):
        import subprocess
        subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref"], check=True)
    # loaded with RTLD_GLOBAL and soname libminkasi.so, so the reference's
    # ctypes.cdll.LoadLibrary("libminkasi.so") fallback resolves to it
    ctypes.CDLL(lib, mode=ctypes.RTLD_GLOBAL)
    install_stubs()
    if REF_ROOT not in sys.path:
        sys.path.insert(0, REF_ROOT)
    import minkasi  # noqa: F401
    return minkasi
