"""Benchmark bookkeeping of the reference's evaluation drivers, host side.

- `.log` / `.info` trajectory files (evaluation/geometric-registration, the
  format of Choi et al.'s ElasticReconstruction tools): records of
  "i j n" followed by a 4x4 transform (or a 6x6 information matrix).
- writeLog.m: a registered pair is logged when its surface overlap on the
  first fragment exceeds 0.30.
- mrEvaluateRegistration.m (external/ElasticReconstruction): recall and
  precision of the logged non-consecutive pairs against the ground truth,
  a pair counting as correct when e^T Info e / Info[0,0] <= 0.04 with
  e = (translation, -quaternion vector part) of gt^-1 * result.
- getError.m (keypoint matching): false-positive rate at 95 % recall over
  1,001 descriptor-distance thresholds.
"""
import numpy as np


def _records(path, rows):
    with open(path) as f:
        lines = [ln for ln in f.read().splitlines() if ln.strip()]
    out = []
    step = rows + 1
    for k in range(0, len(lines) - rows, step):
        head = [int(v) for v in lines[k].split()[:3]]
        mat = np.array([[float(v) for v in lines[k + 1 + r].split()[:rows]] for r in range(rows)])
        out.append((head[0], head[1], head[2], mat))
    return out


def read_log(path):
    """[(i, j, n, 4x4 float64)] from a .log trajectory file."""
    return _records(path, 4)


def read_info(path):
    """[(i, j, n, 6x6 float64)] from a .info file."""
    return _records(path, 6)


def write_log(path, records):
    """writeLog.m's layout: "%d\\t %d\\t %d\\t" then four rows of "%.10f" with tabs."""
    with open(path, "w") as f:
        for i, j, n, rt in records:
            f.write("%d\t %d\t %d\t\n" % (i, j, n))
            for row in np.asarray(rt, np.float64).reshape(4, 4):
                f.write("%.10f\t%.10f\t%.10f\t%.10f\n" % tuple(row))


def write_info(path, records):
    """getGtInfoLog.m's gt.info layout: "%d\t %d\t %d\t" then six rows of "%15.8e"."""
    with open(path, "w") as f:
        for i, j, n, m in records:
            f.write("%d\t %d\t %d\t\n" % (i, j, n))
            for row in np.asarray(m, np.float64).reshape(6, 6):
                f.write("\t ".join("%15.8e" % v for v in row) + "\t\n")


def gt_information(corres_points):
    """getGtInfoLog.m: sum over ground-truth correspondence points q of G^T G,
    G = [I, -[q]x]."""
    q = np.asarray(corres_points, np.float64).reshape(-1, 3)
    M = np.zeros((6, 6))
    for x, y, z in q:
        Qx = np.array([[0.0, -z, y], [z, 0.0, -x], [-y, x, 0.0]])
        G = np.concatenate([np.eye(3), -Qx], 1)
        M += G.T @ G
    return M


def log_records(results, n_fragments, min_overlap=0.30):
    """Pairs to log (writeLog.m): results are (i, j, rt 4x4, overlap on the
    first fragment); kept when the overlap is above min_overlap."""
    return [(i, j, n_fragments, np.asarray(rt, np.float64).reshape(4, 4))
            for i, j, rt, ratio in results if ratio > min_overlap]


def _rotation_quaternion(R):
    """Quaternion (w, x, y, z) of a rotation matrix, the trace branch that
    mrEvaluateRegistration.m's dcm2quat takes for near-identity errors."""
    w = 0.5 * np.sqrt(1.0 + np.trace(R))
    return np.array([w, (R[2, 1] - R[1, 2]) / (4 * w), (R[0, 2] - R[2, 0]) / (4 * w), (R[1, 0] - R[0, 1]) / (4 * w)])


def evaluate_registration(result, gt, gt_info, err2=0.04):
    """(recall, precision) of mrEvaluateRegistration.m over non-consecutive pairs."""
    if not gt:
        return 0.0, 0.0
    index = {(i, j): k for k, (i, j, _, _) in enumerate(gt) if j - i > 1}
    info = {(i, j): m for i, j, _, m in gt_info}
    logged = good = 0
    for i, j, _, rt in result:
        if j - i <= 1:
            continue
        logged += 1
        k = index.get((i, j))
        if k is None:
            continue
        delta = np.linalg.solve(gt[k][3], rt)
        q = _rotation_quaternion(delta[:3, :3])
        e = np.concatenate([delta[:3, 3], q[1:]])
        M = info[(i, j)]
        if float(e @ M @ e) / M[0, 0] <= err2:
            good += 1
    return good / len(index), (good / logged if logged else 0.0)


def fpr_at_95_recall(distances, is_match):
    """getError.m: thresholds 0 .. 1.05 max(distance) in 1,000 steps; a pair
    is predicted a match when its distance is below the threshold; the mean
    false-positive rate over thresholds whose recall is in (0.949, 0.951)."""
    d = np.asarray(distances, np.float64)
    m = np.asarray(is_match).astype(bool)
    top = d.max() * 1.05
    thresh = np.arange(1001) * (top / 1000.0)
    pred = d[None, :] < thresh[:, None]
    tp = (pred & m).sum(1)
    fp = (pred & ~m).sum(1)
    tn = (~pred & ~m).sum(1)
    fn = (~pred & m).sum(1)
    with np.errstate(divide="ignore", invalid="ignore"):
        recall = tp / (tp + fn)
        fpr = fp / (fp + tn)
    sel = (recall > 0.949) & (recall < 0.951)
    return float(np.mean(fpr[sel])) if sel.any() else float("nan")


def read_distance_log(path):
    """getError.m's inputs: a count, then one value per line."""
    v = np.loadtxt(path, dtype=np.float64).reshape(-1)
    return v[1:1 + int(v[0])]
