"""Training labels from the solver's own answers (guided.label_task, host
code over the libpca ABI): given the full canonical set of optimal programs,
every positive state at depth d finishes in K* - d more instructions and
every negative one does not, each checked by the oracle's exhaustive
completion from that state."""
import random

import pytest

from oracle import oracle as O
from pca_gb300 import taskgen
from pca_gb300.guided import label_task
from pca_gb300.pcalib import PCALib


@pytest.mark.parametrize("seed,length", [(2, 2), (16, 3), (18, 4), (50, 4)])
def test_labels_match_exhaustive_completion(seed, length):
    task, _ = taskgen.synthetic_task(seed, length)
    ref, full = O.enumerate_task(task, 3, O.NONE, 1 << 16)
    K = ref.optimal_depth
    if K < 2:
        pytest.skip(f"optimal kernel depth {K}: no inner states to label")
    lib = PCALib()
    states, depth, label, remaining = label_task(lib, task, full, K, random.Random(seed), 4)
    ctx = lib.init_ctx(task)
    assert 1.0 in label and 0.0 in label
    for s, d, y, rem in zip(states, depth, label, remaining):
        assert 1 <= d < K
        # the completion's depth bound counts from the root, as the reference's
        found, n, _, _ = O.exhaustive_complete(ctx, s, K)
        if y == 1.0:
            assert found and n == K - d and rem == K - d
        else:
            assert not found and rem == -1
