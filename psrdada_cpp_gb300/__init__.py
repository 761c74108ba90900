"""GB300-native EDD gated spectrometer (drop-in for psrdada_cpp's GatedSpectrometer).

The compute path is the CUDA library ``libgspec.so`` (C ABI in include/gspec.h);
``gated_spectrometer`` mirrors the reference handler interface over it.
"""
from .gated_spectrometer import (  # noqa: F401
    DadaBufferLayout, RawBytes, GatedSpectrometer, FftSpectrometer, NullSink, CollectingSink, SimpleFileWriter,
    GspecError, GspecConfig, load_library, unpack_device, process_block_noalloc, file_input_stream,
    SINGLE_POL, DUAL_POL, POWER, FULL_STOKES, INTENDED, REFERENCE, FLAG_SATURATION_RECORD,
    FLAG_NO_HOST_BUFFERS, FLAG_UNGATED, GspecInfo, query, tc_dft1024_device, FORM_FP32, FORM_BF16, FORM_FP16,
)
from .serving import Server, Batch, make_config  # noqa: F401
