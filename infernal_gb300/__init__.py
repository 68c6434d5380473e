"""GB300-native QDB scanning CYK / Inside for Infernal covariance models.

Modules: ``lib`` (ctypes binding of the C ABI in include/infernal_gb300.h:
scanners, batches, multi-model launches, calibration, pre-filter), ``cmfile``
(CM reader and configuration, QDB band calculation), ``emit`` (sequences
sampled from a CM), ``pipeline`` (the --nohmm search pipeline), ``prefilter``
(the learned window pre-filter: training and scan-time use),
``profile_case`` (one scan for profiling).
"""
