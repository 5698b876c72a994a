"""pycwb_gb300: PycWB's coherent sky-scan likelihood on GB300 (sm_103a).

The sky loop (DPF regulator + sky scan, pycwb/modules/likelihoodWP) and the
WDM time-delay amplitude build that feeds it (pycwb/utils/td_vector_kernels.py)
run as hand-written CUDA kernels behind the C ABI of include/pycwb_gb300.h;
the Python modules here keep the reference's call signatures.
"""

__version__ = "0.1.0"
