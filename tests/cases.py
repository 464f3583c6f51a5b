"""Small seeded systems shared by the parity tests (sizes the oracle finishes
in seconds)."""
from cipsi_gb300 import synth


def small_cases():
    out = [("small", synth.CONFIGS["small"])]
    specs = [
        # norb, nocc, ranks, ncf, metat, nsym, include_hf, seed
        (14, 4, (1, 2, 3), 80, 2, 1, True, 3),
        (12, 4, (1, 2, 3), 60, 2, 2, True, 4),
        (12, 3, (1, 2, 3, 4), 70, 1, 4, True, 5),
        (12, 4, (2, 3), 50, 2, 2, False, 6),
        (10, 3, (1, 2), 40, 3, 1, False, 7),
    ]
    for i, (norb, nocc, ranks, ncf, metat, nsym, hf, seed) in enumerate(specs):
        out.append((f"mix{i}", synth.SynthConfig(f"mix{i}", norb=norb, nocc=nocc, ncholesky=20, ncf=ncf,
                                                   metat=metat, tau=0.02, ranks=ranks, coef_mode="decay09",
                                                   seed=seed, nsym=nsym, include_hf=hf)))
    return out
