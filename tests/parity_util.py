"""Shared parity helpers of the GPU tests: the NCC error measure and the lockstep comparison
of one sweep (first divergence per line, the mask of matched steps, view-selection checks)."""
import numpy as np

NCC_TOL = 1e-4


def ncc_err(got, want):
    """Error in units of the tolerance: absolute within [0, 2], relative beyond."""
    return np.abs(np.asarray(got, np.float64) - want) / np.maximum(1.0, np.abs(want))


def first_divergence(gd, od, direction, lines=None):
    """Per line of the sweep, the number of leading steps (in processing order) whose depth
    decision matches the oracle's. `lines` restricts the comparison to a range of lines."""
    same = np.abs(gd - od) <= 1e-6 * np.abs(od)
    if direction in (0, 2):       # horizontal sweeps: lines are rows
        by_line = same
    else:                         # vertical sweeps: lines are columns
        by_line = same.T
    if lines is not None:
        by_line = by_line[lines[0]:lines[1]]
    if direction in (2, 3):       # processed from the far end
        by_line = by_line[:, ::-1]
    prefix = np.where(by_line.all(axis=1), by_line.shape[1], np.argmin(by_line, axis=1))
    return prefix, by_line.shape[1]


def matched_mask(shape, prefix, nsteps, direction, line0=0):
    """Pixels of the steps before each line's first divergence (the line's own step
    included when it matched)."""
    mask = np.zeros(shape, bool)
    for i, p in enumerate(prefix):
        line = line0 + i
        steps = np.arange(p)
        if direction in (2, 3):
            steps = nsteps - 1 - steps
        if direction in (0, 2):
            mask[line, steps] = True
        else:
            mask[steps, line] = True
    return mask


def divergence_stats(prefix, nsteps):
    events = int(np.sum(prefix < nsteps))
    decisions = int(np.sum(np.minimum(prefix + 1, nsteps)))
    return events, decisions


def view_selection_mismatches(gvs, ovs, mask):
    """Entries of the view-selection map (S, H, W) that differ on the masked pixels."""
    return int(np.sum(gvs[:, mask] != ovs[:, mask]))
