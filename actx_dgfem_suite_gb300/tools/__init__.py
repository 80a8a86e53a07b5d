"""Command-line tools mirroring ``actx_dgfem_suite/tools``."""
