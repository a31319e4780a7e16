"""The reference's task import path (pyhermes/theory/__init__.py):
``from pyhermes_gb300.theory import Corr_2PCF`` as ``from pyhermes.theory
import Corr_2PCF``."""
from ..corr2pcf import Corr_2PCF
from ..counting import Counting
from ..mc3pcf import Corr_3PCF
from ..multipole import Corr_3PCF_Multipole
from ..projection import SFCProjection

__all__ = ["SFCProjection", "Corr_2PCF", "Corr_3PCF", "Corr_3PCF_Multipole", "Counting"]
