"""GB300-native Paillier engine with HEU ZPaillier (paillier_z) semantics,
and HEU's Okamoto-Uchiyama (ou) scheme on the same kernels.

The compute path is the CUDA library built from ``heu_gb300/csrc`` and
reached through the C-ABI declared in ``include/heu_gb300.h``; there is no
CPU fallback.
"""

import os

# The request server's slots each need their own hardware work queue, or a
# slot's stream waits behind another's kernels (8 queues by default, shared
# round-robin by every stream of the process).  Takes effect if no CUDA
# context exists yet in this process; a value set by the user is kept.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from heu_gb300.capi import HgError, load  # noqa: F401,E402
from heu_gb300.engine import Context, Key, ints_to_limbs, keygen, limbs_to_ints, ou_keygen  # noqa: F401,E402
from heu_gb300.batch import Batch  # noqa: F401,E402
from heu_gb300.server import Server  # noqa: F401,E402
