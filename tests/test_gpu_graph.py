"""Forward + Jacobian replayed as one CUDA graph (crgpu_forward_sens_graph):
bit-identical to the ordinary calls, and a replay reads the conductivities
the buffer holds at that time.  Config 3 (704 systems: two full rounds of
the tensor-core factor and a partial third, which runs on the second
stream) exercises the two-stream recording."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_graph_replay_matches_ordinary_path(gpu_lib):
    import torch

    from titatest_gb300 import MIXED, CRMod, synth
    s = synth.config3()
    g, sv = s.grid, s.survey
    nanz, manz = sv.nanz, g.elanz
    sig = torch.from_numpy(s.sigma.view(np.float64).copy()).cuda()
    volt = torch.zeros(2 * nanz, dtype=torch.float64, device="cuda")
    sens = torch.zeros(2 * nanz * manz, dtype=torch.float64, device="cuda")
    sig2_host = (s.sigma * (1.0 + 0.05 * np.cos(np.arange(manz)))).view(np.float64).copy()
    with CRMod(g, sv, precision=MIXED) as m:
        m.set_stream(torch.cuda.current_stream().cuda_stream)
        m.set_refinement(8, 1e-2)

        def ordinary():
            m.forward_device(sig.data_ptr(), volt.data_ptr())
            m.sens_device(0, sens.data_ptr())
            torch.cuda.synchronize()
            return volt.clone(), sens.clone()

        v0, j0 = ordinary()
        results = []
        for _ in range(3):  # record, then replay twice
            m.forward_sens_graph(sig.data_ptr(), volt.data_ptr(), 0, sens.data_ptr())
            torch.cuda.synchronize()
            results.append((volt.clone(), sens.clone()))
            assert m.stats()["refine_iterations"] >= 1
        for v, j in results:
            assert torch.equal(v, v0) and torch.equal(j, j0)
        # new conductivities in the same buffer: the replay reads them
        sig.copy_(torch.from_numpy(sig2_host).cuda())
        m.forward_sens_graph(sig.data_ptr(), volt.data_ptr(), 0, sens.data_ptr())
        torch.cuda.synchronize()
        v2, j2 = volt.clone(), sens.clone()
        v3, j3 = ordinary()
        assert torch.equal(v2, v3) and torch.equal(j2, j3)
        assert not torch.equal(v2, v0)
