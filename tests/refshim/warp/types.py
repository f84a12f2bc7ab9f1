"""``warp.types`` names the reference uses (float32, array), taken from the
package itself (test infrastructure; see the package docstring)."""


def __getattr__(name):
    import warp

    return getattr(warp, name)
