"""Optimiser description mirroring ``optax.adam``'s signature.

The engine applies Adam itself (the masked ``fbp_adam`` kernel for subdomain
parameters, ``adam_update`` below for the few problem-level parameters); this
callable only records the hyper-parameters, as ``Constants.optimiser`` holds
``optax.adam`` in the reference (fbpinns/constants.py:78-81).
"""

import torch


def adam(learning_rate, b1=0.9, b2=0.999, eps=1e-8, eps_root=0.0):
    return {"name": "adam", "learning_rate": float(learning_rate), "b1": float(b1), "b2": float(b2),
            "eps": float(eps), "eps_root": float(eps_root)}


def adam_update(p, g, m1, m2, count, lr, b1=0.9, b2=0.999, eps=1e-8, eps_root=0.0):
    """In-place Adam on a torch parameter with optax's ordering; count is the
    step count BEFORE this update (shared with the subdomain parameters)."""
    c = count + 1
    m1.mul_(b1).add_((1 - b1) * g)
    m2.mul_(b2).add_((1 - b2) * g * g)
    mh = m1 / (1 - b1 ** c)
    nh = m2 / (1 - b2 ** c)
    p.add_(-lr * (mh / (torch.sqrt(nh + eps_root) + eps)))
