"""morpheus_gb300 -- GB300-native SpMV hot path of the Morpheus sparse library.

Host-side mirror of the reference's container/algorithm API over the C ABI of
libmorpheus_gb300.so (sm_103a kernels).  See include/mgb.h for the ABI and
include/Morpheus_GB300.hpp for the C++ front end.
"""
from .algorithms import dot, dot_async, multiply, multiply_host, reduce, waxpby
from .batched import CsrBatch
from .convert import convert, convert_inplace, from_coo, is_sorted, sort_by_row_and_column, to_coo
from .containers import (COO_FORMAT, CSR_FORMAT, DIA_FORMAT, ELL_FORMAT, HDC_FORMAT, HYB_FORMAT,
                         CSR_ROWS, CSR_ROWS_GATHER, CSR_SEGMENTS, CSR_SPLIT, INVALID_INDEX, NFORMATS, CooMatrix, CsrMatrix, DiaMatrix, DynamicMatrix,
                         EllMatrix, HdcMatrix, HybMatrix, conversion_error_e, formats_e, get_pad_size,
                         matrix_from_host, matrix_to_host)
from .matrix_market import read_matrix_market_file, write_matrix_market_file
from .exceptions import (AllocationException, BadArgumentException, CudaException,
                         FormatConversionException, InvalidInputException, IOException,
                         MorpheusException, NotImplementedException, RuntimeException,
                         TimeoutException)

__all__ = [
    "multiply", "multiply_host", "dot", "dot_async", "reduce", "waxpby",
    "convert", "convert_inplace", "to_coo", "from_coo", "sort_by_row_and_column", "is_sorted",
    "CooMatrix", "CsrMatrix", "DiaMatrix", "EllMatrix", "HybMatrix", "HdcMatrix", "DynamicMatrix",
    "formats_e", "conversion_error_e", "get_pad_size", "matrix_from_host", "matrix_to_host",
    "COO_FORMAT", "CSR_FORMAT", "DIA_FORMAT", "ELL_FORMAT", "HYB_FORMAT", "HDC_FORMAT", "NFORMATS",
    "INVALID_INDEX", "CSR_SEGMENTS", "CSR_ROWS", "CSR_SPLIT", "CSR_ROWS_GATHER",
    "read_matrix_market_file", "write_matrix_market_file",
    "MorpheusException", "NotImplementedException", "FormatConversionException",
    "InvalidInputException", "RuntimeException", "IOException", "CudaException",
    "TimeoutException", "BadArgumentException", "AllocationException",
]
