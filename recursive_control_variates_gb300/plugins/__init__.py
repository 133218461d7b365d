"""Registers the reference's plugin names (plugins/__init__.py:11-17):
integrators ``volpathsimple``, ``twostateprb``, ``meta``, ``cv``,
``twostateprbvolpath`` (plus ``prbvolpath``), the ``twostate`` BSDF and the
``twostatemedium`` medium (registered by ``core``)."""
from ..core import register_integrator
from .cv_integrator import CVIntegrator, MetaIntegrator
from .twostatepath import TwoStatePRBIntegrator
from .twostatevolpath import PRBVolpathIntegrator, TwoStatePRBVolpathIntegrator
from .volpathsimple import VolpathSimpleIntegrator
from .welford import StatisticsEstimator, WelfordVarianceEstimator

register_integrator("twostateprb", TwoStatePRBIntegrator)
register_integrator("meta", MetaIntegrator)
register_integrator("cv", CVIntegrator)
register_integrator("twostateprbvolpath", TwoStatePRBVolpathIntegrator)
register_integrator("prbvolpath", PRBVolpathIntegrator)
register_integrator("volpathsimple", VolpathSimpleIntegrator)

__all__ = [
    "CVIntegrator",
    "MetaIntegrator",
    "TwoStatePRBIntegrator",
    "TwoStatePRBVolpathIntegrator",
    "PRBVolpathIntegrator",
    "VolpathSimpleIntegrator",
    "StatisticsEstimator",
    "WelfordVarianceEstimator",
]
