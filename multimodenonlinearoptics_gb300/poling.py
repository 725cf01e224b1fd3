"""Poling-pattern generators for chi(2) media (host side).

The functions return arrays of domain lengths, the format every solver's ``poling=`` argument and
``setPoling`` take (the engine turns them into per-step orientations, ``src/_NonlinearMedium.cpp:470-503``).
They follow the reference's ``poling.py`` function by function, with the same names, arguments,
errors and outputs, including the corner cases noted per function; the outputs are pinned to the
reference module's own outputs on seeded inputs.  This is setup work on the host: it runs once per
design, before any propagation.
"""

import numpy as np

__all__ = ["periodicPoling", "linearPoling", "linearPolingContinuous", "detunePoling", "dutyCyclePmf",
           "deletedDomainPmf", "threeWaveMismatchRange", "combinePoling", "domainsToSpace"]


def _run_lengths(orientation):
    """Lengths of the maximal runs of equal values in a 1-D array of +/-1."""
    n = orientation.size
    if n == 0:
        return np.zeros(0, dtype=np.int64)
    flips = np.flatnonzero(orientation[1:] != orientation[:-1]) + 1
    return np.diff(np.concatenate(([0], flips, [n])))


def _sampled_domains(phase, dL):
    """Domain lengths of the orientation sign(sin(phase)) sampled every dL (zeros count as +1)."""
    orientation = np.sign(np.sin(phase))
    orientation[orientation == 0.] = 1.
    return _run_lengths(orientation) * dL


def periodicPoling(deltaBeta0, L):
    """Periodic poling that phase matches ``deltaBeta0`` over length L (poling.py:8-14).

    Domains are half a period 2 pi / |deltaBeta0| long, scaled so that they sum to L; the last one
    holds the fractional remainder.  As in the reference, a length that is a whole number of half
    periods leaves a last domain of length zero.
    """
    halfPeriods = 2 * L / (2 * np.pi / abs(deltaBeta0))
    remainder = halfPeriods % 1
    lengths = np.ones(int(halfPeriods) + int(remainder > 0))
    lengths[-1] = remainder
    return lengths * (L / np.sum(lengths))


def linearPoling(k0, kf, L, dL):
    """Chirped poling whose spatial frequency runs linearly from k0 at z=0 to kf at z=L, resolved on a
    grid of step dL (poling.py:17-29).  The orientation is the sign of sin(phi(z)) with
    phi(z) = (kf - k0) z^2 / (2L) + k0 z."""
    z = np.linspace(0, L, int(round(L / dL)))
    return _sampled_domains(0.5 * (kf - k0) * z**2 / L + k0 * z, dL)


def linearPolingContinuous(k0, kf, L):
    """The chirped poling of ``linearPoling`` with exact domain walls (poling.py:32-83).

    The walls are the roots of phi(z) = n pi.  phi(z) is monotonic on [0, L] unless its turning point
    z = -k0 L / (kf - k0) lies inside; then the order n runs to its value at the turning point and
    back, and the root takes the other sign of the quadratic formula's square root past the turn.  A
    turning point where phi is an exact multiple of pi is a double root, kept as one wall.  The last
    root is replaced by L.  (The reference also prints whether that double root occurs; nothing is
    printed here.)
    """
    slope = kf - k0
    nEnd = int((kf + k0) * L / (2 * np.pi))           # order n of the last wall, phi(L) / pi
    zTurn = -k0 * L / slope
    turns = 0 < zTurn < L
    if turns:
        nTurnExact = -k0**2 * L / (2 * np.pi * slope)   # phi(zTurn) / pi
        nTurn = int(nTurnExact)
        double = nTurn == nTurnExact
        stepIn = np.sign(nTurn) if np.sign(nTurn) != 0 else 1
        stepOut = 1 if nEnd > nTurn else -1
        past = 2 if stepOut == np.sign(nEnd) else 1
        orders = np.concatenate([np.arange(0, nTurn, stepIn), double * [nTurn], [0] * (nTurn == 0),
                                 np.arange(nTurn + stepOut * (nTurn != 0), nEnd + past * stepOut, stepOut)])
        split = max(abs(nTurn), 1)
    else:
        step = np.sign(nEnd) if np.sign(nEnd) != 0 else 1
        past = 2 if step == np.sign(nEnd) else 1
        orders = np.arange(0, nEnd + past * np.sign(nEnd), step)
        split = None
    root = np.sqrt((L * k0)**2 + ((2 * np.pi) * orders) * (L * slope))
    if k0 < 0:
        root[:split] *= -1
    elif turns:
        root[split:] *= -1
    if turns and double:
        root[split] = 0
    walls = (root - L * k0) / slope
    walls[-1] = L
    return np.diff(walls)


def detunePoling(kMin, kMax, k0, ka, L, dL):
    """Poling whose spatial frequency follows k(z) = k0 + ka artanh(a (z - z0)), from kMin at z=0 to
    kMax at z=L, on a grid of step dL (poling.py:86-103).  The phase is the integral of k(z)."""
    z = np.linspace(0, L, int(round(L / dL)))
    a = (np.tanh((kMax - k0) / ka) + np.tanh((k0 - kMin) / ka)) / L
    z0 = np.tanh((k0 - kMin) / ka) / a
    phase = ka / (2 * a) * np.log(1 - a**2 * (z - z0)**2) + ka * (z - z0) * np.arctanh(a * (z - z0)) + k0 * z
    return _sampled_domains(phase - phase[0], dL)


def _merge_empty(domains):
    """Drop zero-length domains: the domain after a run of empty ones has the orientation of the one
    before, so it is added to that one.  Returns the index of the last domain kept open."""
    open_ = 0
    pending = False
    for i in range(domains.size - 1):
        if domains[i] == 0:
            pending = True
        elif pending:
            domains[open_] += domains[i]
            domains[i] = 0
            pending = False
        else:
            open_ = i
    return open_


def dutyCyclePmf(nlf, deltaBeta0, L, minSize, normalize=True):
    """Poling whose local duty cycle d(z) = arcsin(nlf(z)) / pi shapes the effective nonlinearity into
    the real function ``nlf`` (poling.py:106-188).

    The periodic poling is taken in domain pairs: the first of each pair is scaled by 2d and the second
    by 2(1-d).  Duty cycles within minSize / (2 half period) of 0 or 1 are clamped there, negative ones
    wrapped by +1.  Each pair's walls are then shifted so that the poled domains stay centred on the
    original grid, and empty domains are merged into their neighbours.
    """
    poling = periodicPoling(deltaBeta0, L)
    pairs = poling.size // 2
    half = poling[0]
    if minSize > poling[0]:
        raise ValueError("minSize larger than half period.")
    minDuty = 0.5 * minSize / poling[0]
    oddCount = poling.size % 2

    strength = nlf(np.linspace(half, L - poling[-1] - half * oddCount, pairs))
    if normalize:
        strength *= 1 / np.max(np.abs(strength))
    elif np.any(np.abs(strength) > 1):
        raise ValueError("Function has value larger than 1")

    duty = np.arcsin(strength) / np.pi
    duty[np.abs(duty) < minDuty] = 0
    duty[np.abs(1 - duty) < minDuty] = 1
    duty[duty < 0] += 1

    out = np.empty_like(poling)
    out[0:2 * pairs:2] = poling[0:2 * pairs:2] * (2 * duty)
    out[1:2 * pairs:2] = poling[1:2 * pairs:2] * (2 * (1 - duty))

    if oddCount:
        # the last, unpaired domain: split it when its duty cycle is wide enough (the reference then
        # restores the last piece to the full remainder, which is mirrored)
        dutyEnd = np.arcsin(nlf(L)) / np.pi
        if dutyEnd >= minDuty and poling[-1] > dutyEnd * poling[0]:
            out[-1] = dutyEnd * poling[0]
            out = np.concatenate([out, [poling[-1] - out[-1]]])
        out[-1] = poling[-1]
    else:
        out[-1] = half + poling[-1] - out[-2]
        if out[-1] < 0:
            out[-2] += out[-1]
            out = out[:-1]

    # centre every poled domain on its original position, relative to the first poled one
    poled = np.flatnonzero(duty)
    first = half * (0.5 - duty[poled[0]])
    for i in poled[1:]:
        shift = half * (0.5 - duty[i]) - first
        out[2 * i - 1] += shift
        out[2 * i + 1] -= shift
    while out[-1] < 0:
        out[-2] += out[-1]
        out = out[:-1]

    open_ = _merge_empty(out)
    if duty[-1] == 0:   # keep the last domain's orientation when its duty cycle is zero
        out[open_] += out[-1]
        out[-1] = 0
    return out[out > 0].copy()


def deletedDomainPmf(nlf, deltaBeta0, L, dutyCycle=0.5, normalize=True, override=False):
    """Poling that shapes the effective nonlinearity into the real function ``nlf`` by deleting domains
    of a periodic poling (poling.py:191-289).

    Each domain pair is a unit of nonlinearity sin(pi dutyCycle).  Units are kept where keeping one
    brings the running sum closer to the (rescaled) cumulative integral of ``nlf``; the kept poled
    domains are joined by the deleted ones.  With a duty cycle other than 0.5 the function must stay
    below the unit unless ``override`` is set.
    """
    if 0 >= dutyCycle or dutyCycle >= 1:
        raise ValueError("Duty cycle not in the open interval (0, 1)")
    if dutyCycle != 0.5 and normalize:
        raise ValueError("Changing the duty cycle and normalizing are incompatible")

    poling = periodicPoling(deltaBeta0, L)
    half = poling[0]
    unpaired = bool(poling.size % 2)
    pairs = poling.size // 2

    if dutyCycle != 0.5:
        if not unpaired:
            lastLength = poling[-1]
        poling[0:2 * pairs:2] *= 2 * dutyCycle
        poling[1:2 * pairs:2] *= 2 * (1 - dutyCycle)
        if not unpaired:
            poling[-1] = lastLength + half - poling[-2]
            if poling[-1] < 0:
                poling[-2] += poling[-1]
                poling = poling[:-1]
                unpaired = True
                pairs -= 1
        elif 2 * dutyCycle * half < poling[-1]:
            # the shortened pairs leave room for one more poled domain at the end
            poling = np.concatenate([poling[:-1], [poling[0], poling[-1] - poling[0]]])
            unpaired = False
            pairs += 1

    units = pairs + unpaired
    strength = nlf(np.linspace(half, L - poling[-1] - half * (poling.size % 2), units))
    if normalize:
        strength *= 1 / np.max(np.abs(strength))
    elif np.any(np.abs(strength) > 1):
        raise ValueError("Function has value larger than 1")

    unit = np.sin(np.pi * dutyCycle)
    if dutyCycle != 0.5 and np.any(unit < strength) and not override:
        raise ValueError("Function takes on values larger than the effective nonlinearity by duty cycle "
                         f"({unit} vs {strength.max()}). "
                         "Combining domain deletion and duty cycle modulation is only allowed when the "
                         "function takes values less than the duty cycle allows. It is suggested that "
                         "the crystal be split up into regions with different design strategies.")

    # greedy matching of the cumulative integral, rescaled to a whole number of units
    target = np.cumsum(strength)
    target *= target[-1] / (unit * np.round(target[-1] / unit))
    total = 0
    keep = np.zeros(strength.size, dtype=bool)
    last = None
    for i in range(target.size - unpaired):
        last = i
        if abs(total + unit - target[i]) < abs(total - target[i]):
            total += unit
            keep[i] = True
    if unpaired:
        # the short last domain is a partial unit; it is compared with the target of the last full pair
        # (the reference reuses the loop's final index here)
        partial = np.sin(0.5 * np.pi * poling[-1] / half)
        if abs(total + partial - target[last]) < abs(total - target[last]):
            total += partial
            keep[-1] = True

    kept = np.flatnonzero(keep)
    poled = half * (2 * dutyCycle)
    startsOn = kept[0] == 0
    endsOn = kept[-1] == units - 1
    out = np.zeros(2 * kept.size + (not startsOn) - (endsOn and unpaired))

    # the reference's final wall index comes from its last loop: the join loop when it ran, else the
    # matching loop above
    j = last
    if startsOn:
        out[0::2] = poled
        for j in range(1, kept.size):
            out[2 * j - 1] = np.sum(poling[2 * kept[j - 1] + 1: 2 * kept[j]])
        if not endsOn:
            out[2 * j + 1] = np.sum(poling[2 * kept[-1] + 1:])
        else:
            out[-1] = poling[-1]
    else:
        out[1::2] = poled
        out[0] = np.sum(poling[0: 2 * kept[0]])
        for j in range(1, kept.size):
            out[2 * j] = np.sum(poling[2 * kept[j - 1] + 1: 2 * kept[j]])
        if not endsOn:
            out[2 * j + 2] = np.sum(poling[2 * kept[-1] + 1:])
        else:
            out[-1] = poling[-1]
    return out


def threeWaveMismatchRange(omega, domega, dbeta0, sign1, sign2,
                           beta1a=0, beta2a=0, beta3a=0,
                           beta1b=0, beta2b=0, beta3b=0,
                           beta1c=0, beta2c=0, beta3c=0):
    """Smallest and largest |wavenumber mismatch| of a three-wave process over a band (poling.py:292-315).

    mismatch(w) = dbeta0 + D_a(w) + sign1 D_b(w) + sign2 D_c(w), D(w) = b1 w + b2 w^2 / 2 + b3 w^3 / 6.
    ``domega`` is a half width (|w| < domega) or a pair (lower, upper) with -lower < w < upper.
    """
    assert abs(sign1) == 1 and abs(sign2) == 1, "Sign must be +/-1"

    def taylor(b1, b2, b3, w):
        return b1 * w + 0.5 * b2 * w**2 + 1/6 * b3 * w**3

    mismatch = dbeta0 + taylor(beta1a, beta2a, beta3a, omega) \
        + sign1 * taylor(beta1b, beta2b, beta3b, omega) \
        + sign2 * taylor(beta1c, beta2c, beta3c, omega)
    if isinstance(domega, (float, int)):
        band = np.abs(omega) < domega
    elif isinstance(domega, (tuple, list, np.ndarray)):
        band = np.logical_and(-domega[0] < omega, omega < domega[1])
    else:
        raise ValueError("unrecognized type for domega")
    inBand = np.abs(mismatch[band])
    return np.min(inBand), np.max(inBand)


class _Merger:
    """Walks two domain-length lists at once and emits the domains of their product (the state of
    ``combinePoling``).  A domain whose orientation repeats the previous one extends it; as in the
    reference, such an extension also clears the remembered orientation, so the next domain is always
    started anew."""

    def __init__(self, a, b):
        self.lists = (a, b)
        self.index = [0, 0]
        self.left = [a[0], b[0]]
        self.sign = [True, True]
        self.prev = False
        self.domains = [0]

    def advance(self, s):
        self.index[s] += 1
        if self.index[s] < self.lists[s].size:
            self.sign[s] ^= True
            self.left[s] = self.lists[s][self.index[s]]
        else:
            self.left[s] = 0

    def emit(self, length):
        orientation = self.sign[0] ^ self.sign[1]
        if orientation == self.prev:
            self.domains[-1] += length
            self.prev = None
        else:
            self.domains.append(length)
            self.prev = orientation


def combinePoling(polingA, polingB, minLength, tol):
    """Product of two poling patterns given as domain lengths (poling.py:318-436).

    Walls closer than ``tol`` are merged, and no domain shorter than ``minLength`` is produced: a short
    remainder is split between its neighbours or absorbed.  When one pattern ends first, the rest of
    the other is appended unchanged.
    """
    m = _Merger(polingA, polingB)
    A, B = 0, 1
    while m.left[A] > 0 and m.left[B] > 0:
        ra, rb = m.left
        if 0 < ra < minLength and 0 < rb < minLength:
            # both short: one domain spanning the longer, the excess carried by the longer list
            m.emit(max(ra, rb))
            excess = abs(ra - rb)
            m.domains[-1] += excess
            longer = A if ra > rb else B
            m.advance(A)
            m.advance(B)
            m.left[longer] += excess
        elif abs(ra - rb) < tol and ra > 0 and rb > 0:
            # walls within tolerance: one wall
            m.emit(min(ra, rb))
            excess = abs(ra - rb)
            longer = A if ra > rb else B
            m.advance(A)
            m.advance(B)
            m.left[longer] += excess
        elif 0 < ra < minLength:
            if rb >= 0.5 * ra + minLength:   # split the short domain between its neighbours
                m.domains[-1] += 0.5 * ra
                m.left[B] -= 0.5 * ra
                m.advance(A)
                m.left[A] += 0.5 * ra
            else:                            # absorb it
                m.domains[-1] += ra
                m.left[B] -= ra
                m.advance(A)
        elif 0 < rb < minLength:
            if ra >= 0.5 * rb + minLength:
                m.domains[-1] += 0.5 * rb
                m.left[A] -= 0.5 * rb
                m.advance(B)
                m.left[B] += 0.5 * rb
            else:
                m.domains[-1] += rb
                m.left[A] -= rb
                m.advance(B)
        elif ra >= rb >= minLength:
            m.emit(rb)
            m.left[A] -= rb
            m.advance(B)
        elif rb > ra >= minLength:
            m.emit(ra)
            m.left[B] -= ra
            m.advance(A)
        elif ra == 0:
            m.emit(rb)
            m.advance(B)
        elif rb == 0:
            m.emit(ra)
            m.advance(A)
        else:
            raise RuntimeError(f"No case applies. remaining A: {ra} remaining B: {rb} minLength: {minLength}")

    if m.index[A] < polingA.size - 1:
        m.domains.extend(polingA[m.index[A]:])
    elif m.index[B] < polingB.size - 1:
        m.domains.extend(polingB[m.index[B]:])
    return np.array(m.domains)


def domainsToSpace(poling, nZSteps):
    """Orientation (+/-1) of each of nZSteps steps for the domain lengths ``poling`` (poling.py:439-471).

    The domains are scaled to nZSteps steps.  A step containing a wall takes the interpolated value
    orientation * (2 frac(wall) - 1), where the orientation is that of the domain the wall ends.
    Vectorised: each step belongs to the first domain whose wall index (the truncated wall position)
    is at or after it.
    """
    poling = np.array(poling)
    if np.any(poling <= 0):
        raise ValueError("Poling contains non-positive length domains")
    walls = np.cumsum(poling, dtype=np.float64)
    walls *= nZSteps / walls[-1]
    wallStep = walls.astype(np.int64)
    firstFree = np.concatenate(([0], wallStep[:-1] + 1))
    if np.any(walls < firstFree):
        raise ValueError("Poling period too small for given resolution")
    steps = np.arange(nZSteps)
    domain = np.searchsorted(wallStep, steps, side="left")
    orientation = np.where(domain % 2 == 0, 1.0, -1.0)
    onWall = wallStep[domain] == steps
    orientation[onWall] *= 2 * np.abs(np.fmod(walls[domain[onWall]], 1)) - 1
    return orientation
