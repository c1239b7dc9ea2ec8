import torch
import torch.library as _tl
_orig = _tl.custom_op
def _custom_op(*args, **kwargs):
    tags = kwargs.get("tags")
    if tags is not None and not isinstance(tags, (tuple, list)):
        kwargs["tags"] = (tags,)
    return _orig(*args, **kwargs)
_tl.custom_op = _custom_op
try:
    from torch._library.custom_ops import CustomOpDef
    CustomOpDef._is_inplace = False
    CustomOpDef._is_out = False
    if not hasattr(CustomOpDef, "_autocast_dtype"):
        CustomOpDef._autocast_dtype = {}
    if not hasattr(CustomOpDef, "_disabled_kernel"):
        CustomOpDef._disabled_kernel = set()
except Exception:
    pass
