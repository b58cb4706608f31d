"""The reference's AI module (src/am/ai), on the GB300 engine: a density-predicting
3-D U-Net (TopOptUNet) and the inference pipeline around it (AIOptimizer).  The
reference declares both and leaves them unimplemented; here the network runs on
the engine's tensor-core convolutions and is trained on the engine's own SIMP
results."""
from .inference import AIOptimizer, run_ai_optimization
from .model import TopOptUNet, load_pretrained

__all__ = ["TopOptUNet", "load_pretrained", "AIOptimizer", "run_ai_optimization"]
