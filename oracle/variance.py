"""Oracle (test infrastructure only): the framebuffer's variance estimate.

Restates Variance_kernel (modules/cpu/fb/frame_ops/Variance.ispc:11-49) and
LiveVarianceFrameOp::getAvgError (fb/frame_ops/Variance.cpp:32-46) on numpy
arrays: per 8x8 render task the mean, over pixels whose
den2 = r + g + b + (1 - a) is positive, of |colour - variance|_1 / sqrt(den2),
times 64; the estimate is the mean of the task errors at or above the
threshold, else the largest task error."""
import numpy as np

TASK = 8


def task_errors(color, variance):
    """color, variance: (H, W, 4) float arrays (rows bottom-up) -> (ty, tx)."""
    c = np.asarray(color, np.float64)
    v = np.asarray(variance, np.float64)
    h, w = c.shape[:2]
    ty, tx = (h + TASK - 1) // TASK, (w + TASK - 1) // TASK
    den2 = c[..., 0] + c[..., 1] + c[..., 2] + (1.0 - c[..., 3])
    ok = den2 > 0
    term = np.where(ok, np.abs(c - v).sum(axis=2) / np.sqrt(np.where(ok, den2, 1.0)), 0.0)
    err = np.zeros((ty, tx))
    for y in range(ty):
        for x in range(tx):
            sl = (slice(y * TASK, (y + 1) * TASK), slice(x * TASK, (x + 1) * TASK))
            cnt = ok[sl].sum()
            err[y, x] = 64.0 * term[sl].sum() / cnt if cnt else 0.0
    return err


def avg_error(err, threshold):
    e = np.asarray(err).ravel()
    act = e[e >= threshold]
    return float(act.mean()) if act.size else float(e.max())


def variance_frame_picks(nframes, seed=43):
    """FrameBuffer::beginFrame (modules/cpu/fb/FrameBuffer.cpp:121-136): of
    every even/odd frame pair, one goes into the variance buffer; on each
    even frame pickOdd = mt() & 1 with std::mt19937 seeded 43
    (FrameBuffer.h:135-137), and frame f accumulates when
    (f even) != pickOdd.  numpy's legacy RandomState is the same Mersenne
    Twister with the same seeding (init_genrand), and its full-range uint32
    draws are the raw outputs."""
    rs = np.random.RandomState(seed)
    picks, pick_odd = [], False
    for f in range(nframes):
        even = (f & 1) == 0
        if even:
            pick_odd = bool(rs.randint(0, 2 ** 32, dtype=np.uint32) & 1)
        picks.append(even != pick_odd)
    return picks


def selected_tasks(err, threshold):
    """LocalFrameBuffer::getRenderTaskIDs (fb/LocalFB.cpp:238-260): the
    tasks whose error exceeds the threshold."""
    return np.asarray(err) > threshold
