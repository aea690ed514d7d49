"""Convergence functions for ``MainLoop`` (idpy/LBM/MultiPhaseLoopChecks.py:37-163).

``CheckUConvergenceSCMP`` uses the device reduction ``sclbm_check_u`` (FP64
accumulation with warp shuffles) instead of a full device-to-host copy.
"""
import numpy as np


def CheckUConvergenceSCMP(lbm, skip_exit_condition=False, print_flag=True):
    first_flag = False
    if 'u_conv' not in lbm.sims_vars:
        lbm.sims_vars['u_conv'], lbm.sims_vars['max_u'] = [], []
        lbm.aux_vars += ['u_conv', 'max_u']
        first_flag = True
    lbm.ComputeMomentsMeta()
    u_conv, max_u = lbm._sim.check_u()
    lbm.sims_vars['u_conv'].append(u_conv)
    lbm.sims_vars['max_u'].append(max_u)
    threshold = 1e-12 if lbm.precision == 'fp64' else 1e-5
    if print_flag and lbm.verbose:
        print('u_conv: ', u_conv, 'max_u: ', max_u)
        print("Conv!", u_conv < threshold, first_flag)
    if skip_exit_condition:
        return False
    return (not first_flag) and u_conv < threshold


def CheckCenterOfMassDeltaPConvergence(lbm):
    first_flag = False
    if 'cm_conv' not in lbm.aux_vars:
        for k in ('cm_conv', 'delta_p', 'p_in', 'p_out', 'is_centered_seq'):
            lbm.sims_vars[k] = []
        lbm.aux_vars += ['cm_conv', 'cm_coords', 'delta_p', 'p_out', 'p_in']
        first_flag = True
    p_in, p_out, delta_p = lbm.DeltaPLaplace()
    break_f = False
    if not first_flag:
        dd = delta_p - lbm.sims_vars['delta_p'][-1]
        chk = [not lbm.sims_vars['is_centered'], abs(delta_p) < 1e-9, abs(dd / delta_p) < 1e-5]
        break_f = any(chk)
    lbm.sims_vars['cm_conv'].append(np.copy(lbm.sims_vars['cm_coords']))
    lbm.sims_vars['delta_p'].append(float(delta_p))
    lbm.sims_vars['p_in'].append(float(p_in))
    lbm.sims_vars['p_out'].append(float(p_out))
    lbm.sims_vars['is_centered_seq'].append(lbm.sims_vars['is_centered'])
    return break_f
