"""sparqsim_gb300 — SparQ's sparse-state gate-application path on GB300.

The operator API mirrors pysparq (same class names, constructor arguments,
conditioned_by_* controls and op(state) / op.dag(state) calls); the state
lives in GPU memory and every operator runs as hand-written sm_103a kernels
behind the C ABI in include/sparq_gb300.h. There is no CPU fallback.
"""
from ._native import SparQError, SparQInvalid, launch_count
from .core import (Boolean, General, Graph, QRAMCircuit_qutrit, Rational, SignedInteger, SparseState,
                   StateStorageType, System, UnsignedInteger, get_clearzero_default_eps,
                   autotune_classes, autotune_reset, get_fwht_arithmetic, get_group_strategy,
                   set_clearzero_default_eps, set_download_engine,
                   set_fwht_arithmetic, set_group_strategy, set_output_sizing)
from .operators import *  # noqa: F401,F403
from .operators import (Abs_SInt, Add_AnyInt_AnyInt_InPlace, Add_ConstUInt_InPlace,
                        Add_Mult_UInt_ConstUInt_InPlace, Add_UInt_ConstUInt, Add_UInt_UInt,
                        Add_UInt_UInt_InPlace, AddRegister, And_UInt_UInt, Assign, BaseOperator,
                        Carry_UInt_UInt, ClearZero, CombineRegister, Compare_UInt_UInt, CondRot_Fixed_Bool,
                        CondRot_General_Bool, Hadamard_Partial, Rot_GeneralUnitary, Hadamard_Int_Batched,
                        NoiseTable, PauliNoise,
                        CondRot_Rational_Bool, Div_UInt_UInt, ElementwiseOperator, FlipBools, Fused,
                        GetMid_UInt_UInt, GlobalPhase, Hadamard_Bool, Hadamard_Int, Hadamard_Int_Full,
                        Init_Unsafe, IsZero_UInt, Less_SInt_SInt, Less_UInt_UInt,
                        Mod_Mult_UInt_ConstUInt_InPlace, Mul_UInt_UInt, MulOverflow_UInt_UInt,
                        Mult_UInt_ConstUInt, Neg_UInt, Negative_SInt, Normalize, Or_UInt_UInt,
                        Overflow_SInt_SInt, Phase_Bool, QRAMLoad, QRAMLoadFast, Reflection_Bool,
                        RemoveRegister, Rot_Bool, RX_Bool, RY_Bool, S_Bool, Select_Bool_UInt_UInt,
                        SelfAdjointOperator, ShiftLeft_InPlace, ShiftRight_InPlace, SplitRegister,
                        Sqrt_UInt, Sub_UInt_UInt, Swap_Bool_Bool, Swap_General_General, T_Bool, X_Bool,
                        Xor_UInt_UInt, Y_Bool, Z_Bool, ZeroConditionalPhaseFlip, add_systems, get_output,
                        synchronize)
from .cks import GetQWRotateAngle_Int_Int_Int
from .cks_qram import SparseMatrix

__all__ = [n for n in dir() if not n.startswith("_")]
