"""pg_gpu_gb300 -- the two-locus linkage-disequilibrium path of pg_gpu on GB300.

Host code mirrors pg_gpu's ``ld_pipeline`` / ``ld_statistics`` /
``haplotype_kernels`` / ``HaplotypeMatrix`` / ``moments_ld`` interfaces; the
compute is libpgld (``include/pgld.h``), hand-written CUDA for sm_103a, called
through ctypes on CUDA device pointers.  There is no CPU path.
"""
from ._lib import PgldError  # noqa: F401
from . import ld_statistics  # noqa: F401
from .genotype_matrix import GenotypeMatrix  # noqa: F401
from .haplotype_matrix import HaplotypeMatrix  # noqa: F401

__version__ = "0.1.0"
