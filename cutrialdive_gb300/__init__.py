"""cutrialdive_gb300 -- GB300-native trial factoring of recurrence-defined sequences.

The hot path (device sieve + per-prime residue propagation) runs as
hand-written CUDA kernels for sm_103a in ``libctd_gpu.so``; this package is
the Python mirror of the reference's library API over its C ABI.
"""
from ._native import CtdError, CtdJob, load as load_native, lib_path  # noqa: F401
from .api import (  # noqa: F401
    PEANO,
    Engine,
    Server,
    dispatch,
    engine,
    factoring_results,
    factors_buffer,
    load_checkpoint,
    make_job,
    num_seq_id,
    num_seq_id_from_string,
    num_seq_spec,
    resume_trial_factoring,
    tf_runtime_options,
    trial_factor,
    trial_factoring_options,
    write_checkpoint,
)

__version__ = "0.1.0"
