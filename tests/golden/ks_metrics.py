"""Spark metrics shared by the reference-ensemble generator
(gen_ks_config1.py) and the GPU distribution test: the definitions of
srs_gb300/metrics.py, applied to both ensembles."""
from srs_gb300.metrics import NAMES, spark_metrics  # noqa: F401
