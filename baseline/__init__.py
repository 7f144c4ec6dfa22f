"""The reference's own binaries, built from a staged copy of its sources: the same-GPU baseline
(ref_gpu.py over the reference's CUDA backend) and the staging recipe (stage.py)."""
