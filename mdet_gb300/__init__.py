"""mdet_gb300 -- GB300 (sm_103a) MetaBAT2 TNF path: tetranucleotide counting,
all-pairs TNF probability, cutoff and per-contig top-k edge selection,
behind the C ABI of include/mdet_tnf.h."""
from .tnf import (Context, Graph, LearnedReport, MdetError, MODES, Network, TrainParams, TrainReport,  # noqa: F401
                  load_library, version)
