"""Per-element sensor traces of a transducer, computed inside the time loop.

``Transducer.post_process_sensor_output`` (fullwave/transducer.py:807-869) turns the per-sensor
traces of a simulation into one trace per active element: the mean over every sensor on the
element's surface (each surface coordinate matched against the sensor coordinates, a sensor
counted once per match), or the trace of the sensor at the surface's middle coordinate.
:func:`element_groups` expresses that as one group id and one weight per sensor, which
``Engine.set_sensor_groups`` applies while recording (``fw_set_sensor_groups``), so a simulation
returns ``[n_out, n_elements]`` directly. :func:`post_process_sensor_output` is the same
operation on recorded per-sensor traces, for checking.
"""

from __future__ import annotations

import numpy as np


def _sensor_index(outcoords):
    index = {}
    for k, c in enumerate(np.asarray(outcoords)):
        index.setdefault(tuple(int(v) for v in c), []).append(k)
    return index


def element_groups(outcoords, element_id_to_element_surface, active_sensor_elements, *,
                   average_surface_signals: bool = True):
    """``(group_of_sensor, weight, n_elements)`` for the active elements in id order."""
    outcoords = np.asarray(outcoords)
    index = _sensor_index(outcoords)
    ids = np.where(np.asarray(active_sensor_elements))[0] + 1
    group = np.full(outcoords.shape[0], -1, dtype=np.int32)
    weight = np.zeros(outcoords.shape[0], dtype=np.float32)
    for g, eid in enumerate(ids):
        surface = np.asarray(element_id_to_element_surface[eid])
        if average_surface_signals:
            members = [k for c in surface for k in index.get(tuple(int(v) for v in c), [])]
        else:
            centre = tuple(int(v) for v in surface[surface.shape[0] // 2])
            members = index[centre][:1]
        if not members:
            raise ValueError(f"element {eid} has no sensor on its surface")
        for k in members:
            if group[k] not in (-1, g):
                raise ValueError(f"sensor {k} lies on the surfaces of two elements")
            group[k] = g
        w = np.float32(1.0 / len(members))
        for k in members:
            weight[k] += w  # a sensor matched twice counts twice, as in the reference
    return group, weight, len(ids)


def post_process_sensor_output(sensor_output, outcoords, element_id_to_element_surface,
                               active_sensor_elements, *, average_surface_signals: bool = True):
    """Host restatement: ``[n_sensors, nt]`` per-sensor traces -> ``[n_elements, nt]``."""
    outcoords = np.asarray(outcoords)
    index = _sensor_index(outcoords)
    ids = np.where(np.asarray(active_sensor_elements))[0] + 1
    out = np.zeros((len(ids), sensor_output.shape[1]), dtype=sensor_output.dtype)
    for g, eid in enumerate(ids):
        surface = np.asarray(element_id_to_element_surface[eid])
        if not average_surface_signals:
            centre = tuple(int(v) for v in surface[surface.shape[0] // 2])
            out[g] = sensor_output[index[centre][0]]
            continue
        n = 0
        for c in surface:
            for k in index.get(tuple(int(v) for v in c), []):
                out[g] += sensor_output[k]
                n += 1
        out[g] /= n
    return out
