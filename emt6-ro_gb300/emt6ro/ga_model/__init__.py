from .model import EMT6RoModel
from .screened import ScreenedModel
