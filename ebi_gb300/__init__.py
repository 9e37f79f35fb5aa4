"""GB300 engine for lemolatoon/ebi's chunked decode-and-query path.

EBI1 columns (Gorilla, Chimp, Chimp128, Elf, ElfOnChimp, BUFF, RLE and
Uncompressed chunks) are kept resident in HBM and decoded by hand-written
sm_103a kernels fused with ebi's operators: materialize, filter to a row
bitmask, sum, min and max.  The
engine is the C ABI of include/ebi_gpu.h (libebi_gpu.so); this package is its
Python mirror of ebi's Decoder / Encoder API.
"""
from . import _native
from .api import (BUFF, CHIMP, Aggregation, AggregationKind, Expr, Op, CHIMP128, ELF, ELF_ON_CHIMP, GORILLA, RLE, SCHEMES, UNCOMPRESSED, Batch, ChunkId,
                  ConversionError,
                  CorruptChunk, CudaError, Decoder, DecoderError, InvalidArgument, IOError_, OutOfMemory,
                  Predicate, PreconditionsNotMet, Range, RangeValue, Server, UnexpectedEndOfChunk, Unsupported,
                  encode, kernel_launches, mask_from_rows, rows_from_mask, run_plain)


def load_library():
    """Loads libebi_gpu.so; raises ImportError when it was not built."""
    return _native.lib()


__all__ = [
    "BUFF", "CHIMP", "CHIMP128", "ELF", "ELF_ON_CHIMP", "GORILLA", "RLE", "SCHEMES", "UNCOMPRESSED", "Batch", "ChunkId", "ConversionError",
    "CorruptChunk", "CudaError", "Decoder", "DecoderError", "InvalidArgument", "IOError_", "OutOfMemory",
    "Predicate", "PreconditionsNotMet", "Range", "RangeValue", "UnexpectedEndOfChunk", "Unsupported", "encode",
    "kernel_launches", "load_library", "Server", "run_plain", "mask_from_rows", "rows_from_mask",
    "Aggregation", "AggregationKind", "Expr", "Op",
]
