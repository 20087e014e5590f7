"""The device-side failure path, exercised without a GPU fault: the tensor-core
transforms' bounded wait for their operand image is made to run out (nsp_debug_inject:
the image copy is not issued, so nothing arrives on the barrier -- a flag that nothing
sets).  The kernels record the fault, skip their tiles, free their tensor memory and
return; the step reports NSP_ERR_DEVICE within seconds, and the same context then steps
exactly like a fresh one."""
import time

import numpy as np
import pytest

from test_gpu_parity import init, nsp, stepper  # noqa: F401  (fixtures)

pytestmark = pytest.mark.gpu


def test_wait_timeout_reports_device_fault_and_context_recovers(nsp):
    u0 = init(nsp, "c0")
    st = stepper(nsp, "c0", nsp.NSP_MIXED)
    assert st.describe()["groups"][0]["theta"] == "tcgen05-3xtf32"
    st.set_state(0, u0)
    st.debug_inject(1)
    t0 = time.perf_counter()
    with pytest.raises(nsp.NspError) as e:
        st.step(1)
    assert time.perf_counter() - t0 < 30.0
    assert e.value.code == nsp.NSP_ERR_DEVICE and "wait ran out" in str(e.value)
    st.debug_inject(0)
    st.set_state(0, u0)
    it = st.step(3)
    got = np.stack(st.get_state(0))
    st.close()
    ref = stepper(nsp, "c0", nsp.NSP_MIXED)
    ref.set_state(0, u0)
    it_ref = ref.step(3)
    assert np.array_equal(got, np.stack(ref.get_state(0)))
    assert np.array_equal(it, it_ref)
    ref.close()
