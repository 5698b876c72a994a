"""GPU drop-ins for pycwb/modules/super_cluster_native: the sub-network-cut sky loop."""

from .sub_net_cut import SUBNET_DTYPE, optimze_sky_loc_from_td, subnet_sky_batched

__all__ = ["SUBNET_DTYPE", "optimze_sky_loc_from_td", "subnet_sky_batched"]
