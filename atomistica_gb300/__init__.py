"""
atomistica_gb300 — GB300-native (CUDA sm_103a) per-step force path of the
Atomistica interatomic-potential library: cell-list neighbour build,
Tersoff / Kumagai / Brenner / Juslin bond-order potentials (FP64 drop-in and
FP32-mixed form), their screened variants TersoffScr / KumagaiScr /
BrennerScr / JuslinScr (FP64) and tabulated (alloy) EAM, behind Atomistica's
potential API.

    from atomistica_gb300 import Tersoff          # ASE-style calculator
    from atomistica_gb300 import native           # _atomistica-style objects

The compute library is libatomistica_gb300.so (C-ABI in
include/atomistica_gb300.h); build it with atomistica_gb300.build.build().
"""

from . import parameters, structures  # noqa: F401
from .parameters import (Albe_PRB_65_195124_PtC, Brenner_PRB_42_9458_C_I,  # noqa: F401
                         Brenner_PRB_42_9458_C_II, Erhart_PRB_71_035211_SiC,
                         Erhart_PRB_71_035211_SiC__Scr, Henriksson_PRB_79_114107_FeC,
                         Juslin_JAP_98_123520_WCH, Juslin_JAP_98_123520_WCH__Scr,
                         Kuopanportti_CMS_111_525_FeCH, Kuopanportti_CMS_111_525_FeCH__Scr,
                         Kioseoglou_PSSb_245_1118_AlN, Kumagai_CompMaterSci_39_457_Si,
                         Kumagai_CompMaterSci_39_457_Si__Scr, Tersoff_PRB_39_5566_Si_C,
                         Tersoff_PRB_39_5566_Si_C__Scr)

__version__ = "0.1.0"


def __getattr__(name):
    # The calculator classes load the CUDA library lazily, so that parameter
    # sets and structure builders stay importable on machines without a GPU.
    if name in ("Atomistica", "Tersoff", "Kumagai", "TersoffScr", "KumagaiScr", "Brenner",
                "BrennerScr", "Juslin", "JuslinScr", "TabulatedEAM", "TabulatedAlloyEAM"):
        from . import calculator
        return getattr(calculator, name)
    if name in ("native", "calculator", "io", "build"):
        import importlib
        return importlib.import_module("." + name, __name__)
    raise AttributeError(name)
