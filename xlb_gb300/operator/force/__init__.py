from xlb_gb300.operator.force.momentum_transfer import MomentumTransfer

__all__ = ["MomentumTransfer"]
