"""Reader of the citizen-state stream file (epi_engine_state_stream_open).

The file holds the reference's per-hour citizen states (CitizenStatesAtHr: every agent's
state letter and cell; engine/src/models/events/citizen_state.rs:27-70) in the compact form
the engine writes on the device:

    header    "EPCS", version, agents, grid                     (u32 x 4)
    keyframe  per agent x, y (u16 x 2), then per agent the letter (u8: s e i r d = 0..4)
    per hour  hour, agents, jumps (u32 x 3); one code byte per agent -- bits 0-3 the Moore
              step since the previous record (0 none, 1..8 = neighbour 0..7 in
              NeighborIterator order, 15 a jump), bits 4-6 the letter; then the jumps
              {agent (u32), x | y << 16 (u32)} in agent order.
"""
from __future__ import annotations

import numpy as np

LETTERS = "seird"
MAGIC = 0x53435045

# NeighborIterator order (engine/src/geography/point.rs:59): row-major 3x3 without the centre
_DX = np.array([0, -1, 0, 1, -1, 1, -1, 0, 1] + [0] * 7, dtype=np.int32)
_DY = np.array([0, -1, -1, -1, 0, 0, 1, 1, 1] + [0] * 7, dtype=np.int32)


def read_state_stream(path: str):
    """Yield (hour, x, y, letters) -- hour 0 for the keyframe, then every recorded hour; x, y
    are int32 arrays and letters uint8 codes (index into LETTERS), one entry per agent."""
    with open(path, "rb") as f:
        head = np.frombuffer(f.read(16), dtype="<u4")
        if len(head) != 4 or head[0] != MAGIC or head[1] != 1:
            raise ValueError(f"{path}: not a citizen-state stream")
        n = int(head[2])
        xy = np.frombuffer(f.read(4 * n), dtype="<u2").reshape(n, 2).astype(np.int32)
        x, y = xy[:, 0].copy(), xy[:, 1].copy()
        letters = np.frombuffer(f.read(n), dtype=np.uint8).copy()
        yield 0, x.copy(), y.copy(), letters.copy()
        while True:
            rec = f.read(12)
            if not rec:
                return
            hour, count, jumps = (int(v) for v in np.frombuffer(rec, dtype="<u4"))
            if count != n:
                raise ValueError(f"{path}: hour {hour} has {count} agents, expected {n}")
            codes = np.frombuffer(f.read(n), dtype=np.uint8)
            step = (codes & 15).astype(np.int64)
            x += _DX[step]
            y += _DY[step]
            if jumps:
                ex = np.frombuffer(f.read(8 * jumps), dtype="<u4").reshape(jumps, 2)
                agents, cell = ex[:, 0].astype(np.int64), ex[:, 1]
                if not (step[agents] == 15).all() or (step == 15).sum() != jumps:
                    raise ValueError(f"{path}: hour {hour}: jump list does not match the codes")
                x[agents] = (cell & 0xFFFF).astype(np.int32)
                y[agents] = (cell >> 16).astype(np.int32)
            letters = (codes >> 4) & 7
            yield hour, x.copy(), y.copy(), letters.copy()


def citizen_uuid(agent: int) -> str:
    """A stable citizen_id for agent index `agent`: the reference draws a random version-4 UUID
    per citizen (Citizen::new, engine/src/citizen/mod.rs:66-75); here the index fills the low 62 bits
    of a version-4, variant-1 UUID, so ids are unique, valid and the same in every run."""
    v = (agent & ((1 << 62) - 1)) | (0x4 << 76) | (0x2 << 62)
    h = f"{v:032x}"
    return f"{h[:8]}-{h[8:12]}-{h[12:16]}-{h[16:20]}-{h[20:]}"


def citizen_states_at_hr(hour: int, x, y, letters) -> dict:
    """One CitizenStatesAtHr record (engine/src/models/events/citizen_state.rs:27-70) as the
    reference's serde_json writes it: {"hr", "citizen_states": [{"citizen_id", "state",
    "location": {"x", "y"}}]}, citizens in agent order."""
    return {"hr": int(hour), "citizen_states": [
        {"citizen_id": citizen_uuid(i), "state": LETTERS[int(l)], "location": {"x": int(a), "y": int(b)}}
        for i, (a, b, l) in enumerate(zip(x, y, letters))]}


def write_citizen_states_json(stream_path: str, out_path: str) -> int:
    """Convert a state-stream file into the reference's message form: one CitizenStatesAtHr JSON
    object per recorded hour, one per line (the payloads the reference's Kafka listener
    publishes on its citizen-states topic, events_kafka_producer.rs:90-99).  Returns the
    number of hours written."""
    import json

    hours = 0
    with open(out_path, "w") as out:
        for hour, x, y, letters in read_state_stream(stream_path):
            if hour == 0:  # the keyframe: the state before the first recorded hour
                continue
            out.write(json.dumps(citizen_states_at_hr(hour, x, y, letters), separators=(",", ":")))
            out.write("\n")
            hours += 1
    return hours
