from xlb_gb300.operator.operator import Operator

__all__ = ["Operator"]
