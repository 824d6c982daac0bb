"""Every C-ABI entry point that queues or waits for GPU work makes its
context's device current for the call and gives the caller's device back
(DeviceScope / AQSG_ON_DEVICE in csrc/aqsg_internal.h), so one host thread
can drive contexts on several GPUs.  Checked on the sources, without a GPU:
each exported definition either opens a device scope, only touches host
state, or hands over to a named function that opens one."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "afquantumsim_gb300" / "csrc"

# entry points that touch no device state (host bookkeeping, plan building
# on the host, or work queued by the server's own worker thread, which makes
# its device current when it starts)
HOST_ONLY = {
    "aqsg_version", "aqsg_last_error", "aqsg_set_exec_mode", "aqsg_set_tensor_cores", "aqsg_set_whole_tile_max",
    "aqsg_ctx_stream",
    "aqsg_launch_count", "aqsg_state_info", "aqsg_check_ops", "aqsg_compile", "aqsg_program_info",
    "aqsg_program_export", "aqsg_program_free", "aqsg_circuit_to_text", "aqsg_circuit_from_text",
    "aqsg_batch_info", "aqsg_batch_tuning", "aqsg_batch_traffic", "aqsg_debug_tile_plan", "aqsg_debug_batch_image",
    "aqsg_debug_ctx_scratch", "aqsg_server_submit", "aqsg_server_start", "aqsg_server_poll",
    "aqsg_server_wait_idle", "aqsg_server_get_stats", "aqsg_noise_trajectory", "aqsg_program_plan",
}
# entry points that hand over to a function which opens the scope
DELEGATES = {
    "aqsg_autotune": "autotune_impl",
    "aqsg_state_prob": "aqsg_state_download_range",
}
SCOPE = re.compile(r"AQSG_ON_DEVICE\(|DeviceScope \w+\(")


def definitions():
    """name -> body text of every `aqsg_*` function definition in csrc."""
    out = {}
    for f in sorted(CSRC.glob("*.cu")):
        s = f.read_text()
        for m in re.finditer(r"^(?:extern \"C\" )?(?:int|size_t|void) (aqsg_\w+|autotune_impl)\([^;{]*\)\s*\{",
                             s, re.M):
            i, depth = m.end(), 1
            while depth:
                depth += {"{": 1, "}": -1}.get(s[i], 0)
                i += 1
            out[m.group(1)] = s[m.end():i]
    return out


def test_every_device_entry_point_opens_a_device_scope():
    defs = definitions()
    exported = [n for n in defs if n.startswith("aqsg_")]
    declared = set(re.findall(r"^\s*(?:int|size_t)\s+(aqsg_\w+)\s*\(",
                              "".join(h.read_text() for h in sorted((ROOT / "include").glob("*.h"))), re.M))
    assert declared == set(exported)  # the scan saw every entry point
    missing = []
    for name in exported:
        if name in HOST_ONLY:
            continue
        body = defs[name]
        if name in DELEGATES:
            target = DELEGATES[name]
            assert target in body, name
            assert SCOPE.search(defs[target]), target
            continue
        if not SCOPE.search(body):
            missing.append(name)
    assert not missing, f"entry points without a device scope: {missing}"


def test_host_only_entry_points_launch_nothing():
    defs = definitions()
    for name in HOST_ONLY & set(defs):
        body = defs[name]
        assert "<<<" not in body and "cudaMemcpy" not in body and "cudaStream" not in body, name


def test_scope_restores_the_callers_device():
    h = (CSRC / "aqsg_internal.h").read_text()
    cls = h[h.index("class DeviceScope"):h.index("#define AQSG_ON_DEVICE")]
    # the destructor sets the previous device back when the constructor switched
    assert "cudaGetDevice(&prev_)" in cls
    assert re.search(r"~DeviceScope\(\)\s*\{\s*if \(switched_\) cudaSetDevice\(prev_\);", cls)
