"""rocket_gb300 -- GB300-native (sm_103a) implementation of Rocket's
phylogenetics all-pair path: K-mer counting, Markov-corrected composition
vectors, and the sparse cosine distance D = (1 - C) / 2 over every pair.

Entry points:
  * the C ABI of libphylogenetics.so (include/phylogenetics.h), a drop-in for
    the reference's JNA-loaded library;
  * ``bindings.Bindings`` / ``kernels.CompositionVectorKernels`` /
    ``context.SequenceAnalysisContext``: Python mirrors of the reference's
    plug-in classes over that ABI;
  * ``engine``: batched construction and the all-pair / query engines.
"""
__all__ = ["bindings", "kernels", "context", "engine", "fasta", "synth"]
