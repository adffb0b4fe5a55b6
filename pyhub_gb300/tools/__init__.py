from .pole import Pole

__all__ = ["Pole"]
