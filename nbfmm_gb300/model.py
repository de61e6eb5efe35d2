"""The reference's initial-condition models (nbfmm::model, include/nbfmm/model/model.hpp:36-233) on the GPU.

Same names and argument order as the reference, so `Stars.initialize(model.generateDisk, n, center, radius,
weight)` works as stars.hpp:111-114 does (initialize appends tick_, cur, prev, weight). Positions are (n, 2)
float32 CUDA tensors (or device addresses), centres (x, y) pairs.
"""
import ctypes

from . import _lib, _check, _ptr, _stream


def _c2(p):
    return (ctypes.c_float * 2)(float(p[0]), float(p[1]))


def generateCircleCenter(num_particle, center_position, radius, weight, center_weight, tick,
                         gpuptr_position_current, gpuptr_position_previous, gpuptr_weight, stream=None):
    _check(_lib.load().nbfmm_model_circle_center(int(num_particle), _c2(center_position), float(radius), float(weight),
                                                 float(center_weight), float(tick), _ptr(gpuptr_position_current),
                                                 _ptr(gpuptr_position_previous), _ptr(gpuptr_weight), _stream(stream)))


def generateCircleUniformCenter(num_particle, center_position, radius, weight, center_weight, tick,
                                gpuptr_position_current, gpuptr_position_previous, gpuptr_weight, stream=None):
    _check(_lib.load().nbfmm_model_circle_uniform_center(
        int(num_particle), _c2(center_position), float(radius), float(weight), float(center_weight), float(tick),
        _ptr(gpuptr_position_current), _ptr(gpuptr_position_previous), _ptr(gpuptr_weight), _stream(stream)))


def generateDisk(num_particle, center_position, radius, weight, tick, gpuptr_position_current,
                 gpuptr_position_previous, gpuptr_weight, stream=None):
    _check(_lib.load().nbfmm_model_disk(int(num_particle), _c2(center_position), float(radius), float(weight),
                                        float(tick), _ptr(gpuptr_position_current), _ptr(gpuptr_position_previous),
                                        _ptr(gpuptr_weight), _stream(stream)))


def generateDiskCenter(num_particle, center_position, radius, weight, center_weight, tick,
                       gpuptr_position_current, gpuptr_position_previous, gpuptr_weight, stream=None):
    _check(_lib.load().nbfmm_model_disk_center(int(num_particle), _c2(center_position), float(radius), float(weight),
                                               float(center_weight), float(tick), _ptr(gpuptr_position_current),
                                               _ptr(gpuptr_position_previous), _ptr(gpuptr_weight), _stream(stream)))


def generateDiskStatic(num_particle, center_position, radius, weight, tick, gpuptr_position_current,
                       gpuptr_position_previous, gpuptr_weight, stream=None):
    _check(_lib.load().nbfmm_model_disk_static(int(num_particle), _c2(center_position), float(radius), float(weight),
                                               float(tick), _ptr(gpuptr_position_current),
                                               _ptr(gpuptr_position_previous), _ptr(gpuptr_weight), _stream(stream)))


def generateDoubleDisk(num_particle1, num_particle2, center_position1, center_position2, radius1, radius2, weight,
                       eccentricity, tick, gpuptr_position_current, gpuptr_position_previous, gpuptr_weight,
                       stream=None):
    _check(_lib.load().nbfmm_model_double_disk(
        int(num_particle1), int(num_particle2), _c2(center_position1), _c2(center_position2), float(radius1),
        float(radius2), float(weight), float(eccentricity), float(tick), _ptr(gpuptr_position_current),
        _ptr(gpuptr_position_previous), _ptr(gpuptr_weight), _stream(stream)))


def generateDoubleDiskCenter(num_particle1, num_particle2, center_position1, center_position2, radius1, radius2,
                             weight, center_weight1, center_weight2, eccentricity, tick, gpuptr_position_current,
                             gpuptr_position_previous, gpuptr_weight, stream=None):
    _check(_lib.load().nbfmm_model_double_disk_center(
        int(num_particle1), int(num_particle2), _c2(center_position1), _c2(center_position2), float(radius1),
        float(radius2), float(weight), float(center_weight1), float(center_weight2), float(eccentricity), float(tick),
        _ptr(gpuptr_position_current), _ptr(gpuptr_position_previous), _ptr(gpuptr_weight), _stream(stream)))


def generateRectangle(num_particle, center_position, width, height, max_weight, tick, gpuptr_position_current,
                      gpuptr_position_previous, gpuptr_weight, stream=None):
    _check(_lib.load().nbfmm_model_rectangle(int(num_particle), _c2(center_position), float(width), float(height),
                                             float(max_weight), float(tick), _ptr(gpuptr_position_current),
                                             _ptr(gpuptr_position_previous), _ptr(gpuptr_weight), _stream(stream)))


def set_uniforms(uniforms=None):
    """Checking hook: take the draws of later model calls from `uniforms` (float32 CUDA tensor, 3 per particle)
    instead of curand; None restores curand. The tensor is kept alive until the next call."""
    global _held_uniforms
    _check(_lib.load().nbfmm_model_set_uniforms(_ptr(uniforms) if uniforms is not None else None))
    _held_uniforms = uniforms


_held_uniforms = None
