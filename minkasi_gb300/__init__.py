"""minkasi_gb300: the minkasi mapmaking hot path on a GB300 (sm_103a).

Drop-in names for the reference's hot-path API (``minkasi.minkasi_all``):
SkyMap, SkyMapCar, PolMap, Mapset, Tod, TodVec, NoiseSmoothedSVD, make_hits, run_pcg,
run_pcg_wprior, map2tod, tod2map_omp, truncate_tod, radec2pix_car, CutsCompact,
tsModel, tsStripes, tsBinnedAz, plus the mixed-precision
solver ``run_pcg_mixed``.  Compute runs in libmkgpu.so (hand-written CUDA,
C ABI in include/mkgpu.h); there is no CPU fallback.
"""
from . import _lib
from ._lib import MkError

_lib.load()  # fail loudly at import if the CUDA library is missing

from .maps import Mapset, SkyMap, SkyMapCar, radec2pix_car  # noqa: E402
from .noise import NoiseSmoothedSVD, smooth_many_vecs  # noqa: E402
from .parallel import barrier, have_mpi  # noqa: E402
from .polmap import PolMap  # noqa: E402
from .tsmodels import CutsCompact, tsBinnedAz, tsModel, tsStripes  # noqa: E402
from .pcg import null_precon, run_pcg, run_pcg_mixed, run_pcg_wprior  # noqa: E402
from .projections import jacobi_precon, make_hits, map2tod, tod2map_omp, tod2map_simple  # noqa: E402
from .tods import Tod, TodVec  # noqa: E402
from .truncate import find_good_fft_lens, truncate_tod  # noqa: E402

__all__ = ["Mapset", "SkyMap", "SkyMapCar", "PolMap", "CutsCompact", "tsModel", "tsStripes", "tsBinnedAz", "radec2pix_car", "NoiseSmoothedSVD", "smooth_many_vecs", "barrier", "have_mpi",
           "null_precon", "run_pcg", "run_pcg_mixed", "run_pcg_wprior", "jacobi_precon", "make_hits",
           "map2tod", "tod2map_omp", "tod2map_simple", "Tod", "TodVec", "find_good_fft_lens",
           "truncate_tod", "MkError"]
