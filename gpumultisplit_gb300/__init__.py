"""gpumultisplit_gb300: stable multisplit, multisplit radix sort, histogram and
two-bucket compaction for NVIDIA GB300 (sm_103a), behind a C ABI
(include/gpumultisplit.h) and a host API that mirrors owensgroup/GpuMultisplit.
"""
from .api import (  # noqa: F401
    BucketIdentifier,
    bits_bucket,
    compaction_allocate_key_only,
    compaction_allocate_key_value,
    compaction_context,
    compaction_key_only,
    compaction_key_value,
    compaction_release_memory,
    delta_bucket,
    delta_func,
    even_float_bucket,
    histogram_even,
    histogram_range,
    mask_bucket,
    ms_bucket_sort_4bit,
    ms_bucket_sort_7bit,
    ms_sort_context,
    multisplit_allocate_key_only,
    multisplit_allocate_key_value,
    multisplit_context,
    multisplit_histogram,
    multisplit_key_only,
    multisplit_key_value,
    multisplit_release_memory,
    multisplit_sort_7bit,
    multisplit_sort_7bit_allocate,
    multisplit_sort_7bit_allocate_pairs,
    multisplit_sort_7bit_pairs,
    multisplit_sort_release_memory,
    multisplit_stages,
    range_bucket,
    read_device_error,
    set_sort_method,
    sort_method,
    test_bucket,
)
from ._lib import GmsError, load  # noqa: F401
from .api import (  # noqa: F401
    multisplit_sort_4bit, multisplit_sort_4bit_allocate, multisplit_sort_4bit_allocate_pairs, multisplit_sort_4bit_pairs,
    multisplit_sort_5bit, multisplit_sort_5bit_allocate, multisplit_sort_5bit_allocate_pairs, multisplit_sort_5bit_pairs,
    multisplit_sort_6bit, multisplit_sort_6bit_allocate, multisplit_sort_6bit_allocate_pairs, multisplit_sort_6bit_pairs,
    multisplit_sort_8bit, multisplit_sort_8bit_allocate, multisplit_sort_8bit_allocate_pairs, multisplit_sort_8bit_pairs,
    multisplit_sort_bits, multisplit_sort_bits_allocate, multisplit_sort_bits_pairs,
    multisplit_histogram_wide, multisplit_sort_wide, multisplit_sort_wide_allocate, multisplit_wide,
    multisplit_wide_allocate,
)
from .batched import (  # noqa: F401
    BatchedMultisplit,
    Segment,
    autotune,
    reset_tuning,
    set_tuning,
    tile_variant_shape,
    tuning_table,
)
from .serving import Result, Server  # noqa: F401
