"""CPU oracle of CUDIMOT's data loading steps (test infrastructure).

remove_nonpositive restates dMRI_Data<T>::remove_NonPositive_entries
(dMRI_Data.cu:15-30) step by step, for one voxel's signals at a time, as
dMRI_Data::getMeasPart applies it to every voxel when --rician is set
(dMRI_Data.cu:133):

    float MinS = Voxdata.Minimum1(pos);   float MaxS = Voxdata.Maximum();
    if (MinS <= 0 && MaxS > 0) {
      while (MinS <= 0) { remember pos; Voxdata(pos) = MaxS; MinS = Minimum1(pos); }
      MinS = Voxdata.Minimum();
      every remembered entry = MinS;
    }

MinS and MaxS are floats, so the comparisons and the values written are
float-rounded, and Minimum1 returns the first position of the minimum.
"""
import numpy as np


def _f32(x):
    return float(np.float32(x))


def remove_nonpositive_voxel(v):
    v = np.array(v, dtype=np.float64)
    pos = int(np.argmin(v))          # Minimum1: first position of the minimum
    mins = _f32(v[pos])
    maxs = _f32(v.max())
    if mins <= 0 and maxs > 0:
        minpositions = []
        while mins <= 0:
            minpositions.append(pos)
            v[pos] = maxs            # temporarily the maximum
            pos = int(np.argmin(v))
            mins = _f32(v[pos])
        mins = _f32(v.min())
        for p in minpositions:
            v[p] = mins
    return v


def remove_nonpositive(meas):
    """meas [nvox][nmeas] -> a cleaned copy."""
    meas = np.asarray(meas, dtype=np.float64)
    return np.stack([remove_nonpositive_voxel(r) for r in meas]) if len(meas) else meas.copy()
