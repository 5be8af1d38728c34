"""Host-side behaviour of the drop-in registrator that needs no GPU."""
import numpy as np

from zorro_gb300.registrator import ImageRegistrator, copy_config


def test_masks_default_none():
    assert ImageRegistrator().masks is None


def test_masks_after_registration_are_the_all_true_mask_made_on_first_read():
    # what a registration without a mask leaves (zorro.py:584-586): the
    # engine records the shape, the array is made when read
    r = ImageRegistrator()
    r._ones_mask_shape = (6, 7)
    assert "_masks" in vars(r) and vars(r)["_masks"] is None
    m = r.masks
    assert m.shape == (1, 6, 7) and m.dtype == bool and m.all()
    assert r.masks is m  # made once


def test_masks_set_by_the_user_stay():
    r = ImageRegistrator()
    r._ones_mask_shape = (6, 7)
    user = np.zeros((6, 7), dtype=bool)
    r.masks = user
    assert r.masks is user
    r.masks = None
    assert r.masks is None


def test_copy_config_does_not_carry_masks():
    r = ImageRegistrator()
    r.masks = np.ones((3, 3), dtype=bool)
    r.maxShift = 55
    d = copy_config(r, ImageRegistrator())
    assert d.masks is None and d.maxShift == 55
