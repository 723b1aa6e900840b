"""sable_gb300 — GB300 (sm_103a) VBR SpMV / SpMM with SABLE's API surface.

Reference-named entry points (reikdas/SABLE):
    VBR                                 src/vbr.py
    read_vbr, read_vbrc, write_vbr_matrix, write_dense_vector,
    write_dense_matrix                  utils/fileio.py
    convert_vbr_to_compressed, convert_sparse_to_vbr
                                        utils/convert_real_to_vbr.py
    vbr_spmv_codegen, vbr_spmm_codegen, gen_single_threaded_spmv,
    gen_multi_threaded_spmv, gen_single_threaded_spmm,
    gen_multi_threaded_spmm             src/codegen.py
    vbr_matrix_gen                      synthesize_matrices/vbr_matrices_gen.py
The compute path is libsable.so (CUDA, sm_103a) only.
"""
from .vbr import VBR
from .synth import vbr_matrix_gen
from .fileio import (read_vbr, read_vbrc, write_vbr_matrix, write_dense_vector, write_dense_matrix,
                     read_vector, read_matrix, write_mm_file)
from .convert import convert_vbr_to_compressed, convert_sparse_to_vbr

__all__ = ["VBR", "read_vbr", "read_vbrc", "write_vbr_matrix", "write_dense_vector", "write_dense_matrix",
           "read_vector", "read_matrix", "write_mm_file", "convert_vbr_to_compressed", "convert_sparse_to_vbr",
           "vbr_matrix_gen"]
