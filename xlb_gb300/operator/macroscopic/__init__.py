from xlb_gb300.operator.macroscopic.macroscopic import Macroscopic

__all__ = ["Macroscopic"]
