"""GB300-native projector-DQMC sweep for KAPDQMC's t-U, t-V and t-UV models."""
from .geometry import area_index, i_xy, nn2idx, nnidx_F, nnK_Matrix, xy_i  # noqa: F401
from .model import (Initial_s, tU_Hubbard_Para, tU_Hubbard_Para_,  # noqa: F401
                    tUV_Hubbard_Para, tUV_Hubbard_Para_, tV_Hubbard_Para,
                    tV_Hubbard_Para_)
