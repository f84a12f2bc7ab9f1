"""``import warp.torch`` (warp_utils.py:2): the torch interop lives on the
package itself here (to_torch / from_torch)."""
